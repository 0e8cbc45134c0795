/*
 * CPU oracle for the UFEMISM ice-velocity solve -- TEST INFRASTRUCTURE ONLY.
 *
 * A literal FP64 C restatement of the reference Fortran routines on the SSA/SIA path,
 * following their loop order and expression order (built with -ffp-contract=off so no
 * fused multiply-adds change the rounding). Arrays use the reference's own layout: 1-based
 * index values, column-major 2-D arrays, unused neighbour slots 0. The reference itself is
 * Fortran 90 + MPI + netCDF and cannot be compiled where this oracle is built, and it ships
 * no tests or golden vectors, so parity of this restatement is pinned only by its own
 * known-answer tests (linear-field exactness of the neighbour functions, the colouring
 * invariant, the analytic SIA dome) and by reading: "parity unpinned" against the
 * reference binary.
 *
 * Only tests, the package smoke check and the CPU-baseline leg of the benchmark may call
 * into this library; it is never the product path.
 */
#ifndef UFE_ORACLE_H
#define UFE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes (mirror of the reference's MPI_ABORT sites). */
enum {
  OR_OK = 0,
  OR_NOT_CONVERGED = 1,        /* SOR hit SSA_max_inner_loops (reference: warning) */
  OR_RESET_ONCE = 2,           /* one reset to zero happened, then converged */
  OR_ERR_DIVERGED = -1,        /* second reset: reference calls MPI_ABORT */
  OR_ERR_BAD_MESH = -2,        /* make_combined_AaAc_mesh could not find an Ac vertex */
  OR_ERR_COLOUR_IDENTIFY = -3, /* five-colouring reached 'identify' (reference aborts) */
  OR_ERR_COLOUR_STUCK = -4,    /* reduce / colour 'got stuck' */
  OR_ERR_COLOUR_QUEUE = -5,    /* queue-consistency abort in the colouring */
  OR_ERR_COLOUR_INVALID = -6,  /* check_solution failed */
  OR_ERR_BAD_ARG = -7,
};

/* Base triangulation (inputs to make_Ac_mesh), reference type_mesh fields. */
typedef struct or_base {
  int32_t nV, nTri, nC_mem;
  const double *V;          /* (nV,2) */
  const int32_t *nC;        /* (nV) */
  const int32_t *C;         /* (nV,nC_mem) */
  const int32_t *niTri;     /* (nV) */
  const int32_t *iTri;      /* (nV,nC_mem) */
  const int32_t *Tri;       /* (nTri,3) */
  const int32_t *edge_index;/* (nV) */
} or_base;

/* Everything make_Ac_mesh, get_neighbour_functions and the colouring produce.
 * Caller allocates: nAc = nV + nTri - 1 (Euler), nVAaAc = nV + nAc. */
typedef struct or_aaac {
  int32_t nAc, nVAaAc;
  /* Aa neighbour functions (get_neighbour_functions) */
  double *Nx, *Ny, *Nxx, *Nxy, *Nyy;  /* (nV,nC_mem+1) */
  /* Ac mesh */
  int32_t *iAci;            /* (nV,nC_mem) */
  int32_t *Aci;             /* (nAc,4) */
  double *VAc;              /* (nAc,2) */
  double *Nx_Ac, *Ny_Ac, *No_Ac; /* (nAc,4) */
  double *Np_Ac;            /* (nAc) */
  int32_t *edge_index_Ac;   /* (nAc) */
  /* combined AaAc mesh */
  double *VAaAc;            /* (nVAaAc,2) */
  int32_t *nCAaAc;          /* (nVAaAc) */
  int32_t *CAaAc;           /* (nVAaAc,nC_mem) */
  double *Nx_AaAc, *Ny_AaAc, *Nxx_AaAc, *Nxy_AaAc, *Nyy_AaAc; /* (nVAaAc,nC_mem+1) */
  /* five-colouring */
  int32_t *colour;          /* (nVAaAc) */
  int32_t *colour_vi;       /* (nVAaAc,5) */
  int32_t *colour_nV;       /* (5) */
} or_aaac;

/* mesh_ArakawaC_module.f90:24-540 + mesh_derivatives_module.f90:14-75 */
int or_build_aaac(const or_base *b, or_aaac *m);
/* mesh_five_colour_module.f90:18-137; identify_count receives how often the Q5 branch
 * found a pair (the reference aborts at the first). */
int or_five_colouring(const or_base *b, or_aaac *m, int32_t *reduce_iterations);

/* Neighbour functions of one vertex (mesh_derivatives_module.f90:76-313), exposed for
 * known-answer tests. V_vc is (nC_mem,2) column-major with ld = ld_vc. */
void or_neighbour_functions_vertex(const double *V_vi, int n, const double *V_vc, int ld_vc,
                                   int is_edge, double *Nx, double *Ny, double *Nxx,
                                   double *Nxy, double *Nyy);

/* Physics parameters and SSA/SIA knobs (parameters_module.f90:9-21,
 * configuration_module.f90:124-126,169-184). */
typedef struct or_params {
  double SSA_RN_tol;
  int32_t SSA_max_outer_loops;
  double SSA_max_residual_UV;
  double SSA_SOR_omega;
  int32_t SSA_max_inner_loops;
  double m_enh_ssa, m_enh_sia;
  int32_t sliding_law;            /* 0 = Coulomb_regularised, 1 = linear (S = beta^2) */
  int32_t use_analytical_GL_flux;
  int32_t zero_velocities;        /* benchmark experiments that skip the SSA */
  int32_t nZ;
  const double *zeta;             /* (nZ) */
  int32_t n_threads;              /* OpenMP threads over rows of one colour (1 = serial) */
  /* Replay: if >0, run exactly this many Picard iterations, and per Picard iteration the
   * SOR sweep counts in replay_sweeps (ignores the tolerances). */
  int32_t replay_picard;
  const int32_t *replay_sweeps;
  /* If non-null, the solve stores its running total of SOR sweeps here after every sweep
   * (read by a benchmark thread to time consecutive pieces of one solve). */
  volatile int64_t *progress;
} or_params;

/* Ice fields read / written by solve_SSA (type_ice_model, data_types_module.f90:15-214). */
typedef struct or_ssa_fields {
  /* Aa (nV) */
  const double *Hi, *Hb, *SL, *dHs_dx_shelf, *dHs_dy_shelf, *A_flow_mean;
  const int32_t *mask_sheet;
  /* Ac (nAc) */
  const double *Hi_Ac, *Hb_Ac, *SL_Ac, *dHs_dx_shelf_Ac, *dHs_dy_shelf_Ac, *A_flow_mean_Ac;
  /* linear sliding law: beta^2 per AaAc vertex (nVAaAc), or NULL with beta_sq_const */
  const double *beta_sq_AaAc;
  double beta_sq_const;
  /* GL flux inputs (only with use_analytical_GL_flux) */
  const int32_t *mask_gl_Ac;        /* (nAc) */
  const double *dHi_dx_Ac, *dHi_dy_Ac, *dSL_dx_Ac, *dSL_dy_Ac, *dHb_dx_Ac, *dHb_dy_Ac; /* (nAc) */
  /* in/out: warm start and result */
  double *U_SSA, *V_SSA;            /* (nV) */
  double *Ux_SSA_Ac, *Uy_SSA_Ac;    /* (nAc) */
  double *N_AaAc;                   /* (nVAaAc) Picard state, persists between calls */
  /* out */
  double *Up_SSA_Ac, *Uo_SSA_Ac;    /* (nAc) */
  double *eta_AaAc, *S_AaAc, *tau_c_AaAc, *phi_fric_AaAc; /* (nVAaAc) */
} or_ssa_fields;

typedef struct or_ssa_stats {
  int32_t picard_iterations;        /* viscosity iterations entered */
  int32_t linear_solves;
  int64_t total_sweeps;
  int32_t resets;
  int32_t not_converged;            /* linear solves that hit SSA_max_inner_loops */
  double last_RN;
  double last_max_residual;
  int32_t sweeps[64];               /* SOR sweeps per linear solve (first 64) */
} or_ssa_stats;

int or_solve_SSA(const or_base *b, const or_aaac *m, const or_params *p, or_ssa_fields *f,
                 or_ssa_stats *st);

/* One linear SOR solve with given eta/S (solve_SSA_linearised), for unit tests. The
 * AaAc-gathered fields are passed directly. */
int or_solve_SSA_linearised(const or_base *b, const or_aaac *m, const or_params *p,
                            const double *Hi, const double *Hb, const double *SL,
                            const double *hx, const double *hy, const double *eta,
                            const double *S, const int32_t *mask_gl_Ac,
                            double *U, double *V, int32_t *sweeps, double *max_res);

/* SIA (ice_dynamics_module.f90:240-314). */
typedef struct or_sia_fields {
  const int32_t *mask_sheet_Ac;     /* (nAc) */
  const double *Hi_Ac, *dHs_dx_Ac, *dHs_dy_Ac, *dHs_dp_Ac, *dHs_do_Ac; /* (nAc) */
  const double *A_flow_Ac;          /* (nAc,nZ) */
  double *D_SIA_3D_Ac;              /* (nAc,nZ) */
  double *D_SIA_Ac, *Ux_SIA_Ac, *Uy_SIA_Ac, *Up_SIA_Ac, *Uo_SIA_Ac; /* (nAc) */
  double *U_SIA, *V_SIA, *D_SIA;    /* (nV) */
} or_sia_fields;

int or_solve_SIA(const or_base *b, const or_aaac *m, const or_params *p, or_sia_fields *f);

/* Input preparation: the part of update_general_ice_model_data that feeds the solve
 * (general_ice_model_data_module.f90:23-96 without temperature/flow-factor physics). */
typedef struct or_geom {
  const double *Hi, *Hb, *SL;       /* (nV) */
  /* outputs, Aa (nV) */
  double *Hs, *dHi_dx, *dHi_dy, *dHs_dx, *dHs_dy, *dHs_dx_shelf, *dHs_dy_shelf;
  int32_t *mask_ocean, *mask_ice, *mask_sheet, *mask_shelf;
  /* outputs, Ac (nAc) */
  double *Hi_Ac, *Hb_Ac, *SL_Ac, *Hs_Ac;
  double *dHi_dx_Ac, *dHi_dy_Ac, *dHi_dp_Ac, *dHi_do_Ac;
  double *dHb_dx_Ac, *dHb_dy_Ac, *dHb_dp_Ac, *dHb_do_Ac;
  double *dHs_dx_Ac, *dHs_dy_Ac, *dHs_dp_Ac, *dHs_do_Ac;
  double *dSL_dx_Ac, *dSL_dy_Ac, *dSL_dp_Ac, *dSL_do_Ac;
  double *dHs_dx_shelf_Ac, *dHs_dy_shelf_Ac;
  int32_t *mask_ocean_Ac, *mask_ice_Ac, *mask_sheet_Ac, *mask_shelf_Ac, *mask_gl_Ac;
} or_geom;

int or_update_geometry(const or_base *b, const or_aaac *m, or_geom *g);

/* calculate_ice_thickness_change (ice_dynamics_module.f90:31-237); Cw and dVi_in are
 * (nV, nC_mem); zero_edges applies the domain-edge rule (every configuration except the
 * SSA_icestream benchmark); mask_noice may be NULL. Hi is updated in place. */
int or_thickness_change(const or_base *b, const or_aaac *m, const double *A, const double *Cw,
                        const double *Up_SIA_Ac, const double *Up_SSA_Ac, const double *SMB_year,
                        const double *BMB, const int32_t *mask_noice, double dt, int zero_edges,
                        double *Hi, double *Hi_prev, double *dHi_dt, double *dVi_in);

/* solve_SIA_3D (ice_dynamics_module.f90:317-405); A_flow and the outputs are (nV, nZ). */
int or_solve_SIA_3D(const or_base *b, const or_aaac *m, const double *zeta, int nZ, double m_enh_sia,
                    const double *Hi, const int32_t *mask_shelf, const int32_t *mask_sheet, const double *dHs_dx,
                    const double *dHs_dy, const double *dHi_dx, const double *dHi_dy, const double *A_flow,
                    const double *dHb_dt, const double *U_SSA, const double *V_SSA, double *U_3D, double *V_3D,
                    double *W_3D);

/* bottom_frictional_heating (thermodynamics_module.f90:281-311) on the Aa vertices. */
void or_frictional_heating(int nV, const int32_t *mask_sheet, const double *tau_c_AaAc, const double *U,
                           const double *V, double *heating);

/* ice_physical_properties (general_ice_model_data_module.f90:298-462). flow_law 0: the
 * Arrhenius law from Ti (nV, nZ), Ti_Ac = map_Aa_to_Ac_3D(Ti); 1: the EISMINT-type benchmarks
 * (constant A, Ki, Cpi; Ti not read); 2: MISMIP_mod (A from the time; only the A fields
 * written). 2-D arrays are (nV, nZ) and (nAc, nZ), column-major. */
int or_ice_physical_properties(int nV, int nAc, int nZ, const double *zeta, const int32_t *Aci, int flow_law,
                               double time, const double *Hi, const int32_t *mask_sheet,
                               const int32_t *mask_sheet_Ac, const double *Ti, double *A_flow, double *A_flow_Ac,
                               double *A_flow_mean, double *A_flow_mean_Ac, double *Ti_pmp, double *Cpi, double *Ki,
                               double *Ti_Ac);

/* The triangle functions NxTri/NyTri (nTri,3) of get_neighbour_functions
 * (mesh_derivatives_module.f90:30-47) and the vertex resolution mesh%R
 * (mesh_help_functions_module.f90:195-211; domain_width = xmax - xmin). */
void or_triangle_functions(const or_base *b, double *NxTri, double *NyTri);
void or_vertex_resolution(const or_base *b, double domain_width, double *R);
/* get_upwind_derivative_vertex_3D (mesh_derivatives_module.f90:434-483) for every vertex and
 * layer; U, V, d, ddx, ddy are (nV, nZ). Returns the number of (vertex, layer) pairs without an
 * upwind triangle (their derivatives are 0 here; the reference reads outside NxTri there). */
long long or_upwind_derivatives_3d(const or_base *b, const or_aaac *m, int nZ, const double *R, const double *NxTri,
                                   const double *NyTri, const double *U, const double *V, const double *d,
                                   double *ddx, double *ddy);

/* determine_masks in full (general_ice_model_data_module.f90:97-297). aa is (nV, OR_MASK_COUNT)
 * and ac (nAc, OR_MASK_COUNT), column-major, columns in the order below; the TYPE column holds
 * the combined type (0 land, 1 ocean, 2 lake, 3 sheet, 4 shelf, 5 coast, 6 margin, 7 grounding
 * line, 8 calving front). Hi_Ac, Hb_Ac, SL_Ac are the Aa-to-Ac maps of Hi, Hb, SL. */
enum {
  OR_MASK_LAND = 0, OR_MASK_OCEAN, OR_MASK_LAKE, OR_MASK_ICE, OR_MASK_SHEET, OR_MASK_SHELF, OR_MASK_COAST,
  OR_MASK_MARGIN, OR_MASK_GL, OR_MASK_CF, OR_MASK_TYPE, OR_MASK_COUNT
};
void or_determine_masks(const or_base *b, const or_aaac *m, const double *Hi, const double *Hb, const double *SL,
                        const double *Hi_Ac, const double *Hb_Ac, const double *SL_Ac, int32_t *aa, int32_t *ac);

/* Primitive operators, for tests. */
void or_map_Aa_to_Ac(const or_aaac *m, int nV, const double *d_Aa, double *d_Ac);
void or_map_Ac_to_Aa(const or_base *b, const or_aaac *m, const double *d_Ac, double *d_Aa);
void or_ddx_ddy_AaAc(const or_aaac *m, int nC_mem, const double *d, double *ddx, double *ddy);
void or_neumann_AaAc(const or_base *b, const or_aaac *m, double *d);

#ifdef __cplusplus
}
#endif
#endif
