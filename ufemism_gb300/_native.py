"""ctypes declarations of the C-ABI in include/ufemism_gb300.h.

The shared library is built in-tree (``ufemism_gb300/_build/libufemism_gb300.so``). There is
no CPU fallback: loading fails loudly if the library is missing, and every solve reports
UFE_NO_DEVICE without a usable sm_103a GPU.
"""
from __future__ import annotations

import ctypes as ct
import os

from . import build as _build

P = ct.c_void_p
I32 = ct.c_int32
F64 = ct.c_double

UFE_OK, UFE_NOT_CONVERGED, UFE_RESET_ONCE = 0, 1, 2
UFE_DIVERGED, UFE_BAD_MESH, UFE_COLOUR_IDENTIFY, UFE_TIMEOUT = -1, -2, -3, -4
UFE_CUDA_ERROR, UFE_BAD_ARG, UFE_NO_DEVICE, UFE_OUT_OF_MEMORY = -5, -6, -7, -8
UFE_FP64, UFE_MIXED = 0, 1
UFE_SIA_NOALLOC_MAX_AC = 262144   # scratch limit of ufe_sia_solve_noalloc (Ac edges)
UFE_SLIDING_COULOMB_REGULARISED, UFE_SLIDING_LINEAR = 0, 1

STATUS_NAMES = {0: "UFE_OK", 1: "UFE_NOT_CONVERGED", 2: "UFE_RESET_ONCE", -1: "UFE_DIVERGED",
                -2: "UFE_BAD_MESH", -3: "UFE_COLOUR_IDENTIFY", -4: "UFE_TIMEOUT", -5: "UFE_CUDA_ERROR",
                -6: "UFE_BAD_ARG", -7: "UFE_NO_DEVICE", -8: "UFE_OUT_OF_MEMORY"}


class MeshDesc(ct.Structure):
    _fields_ = [("nV", I32), ("nAc", I32), ("nVAaAc", I32), ("nC_mem", I32)] + \
               [(n, P) for n in ("V", "nC", "iAci", "Aci", "edge_index", "edge_index_Ac", "nCAaAc", "CAaAc",
                                 "Nx_AaAc", "Ny_AaAc", "Nxx_AaAc", "Nxy_AaAc", "Nyy_AaAc", "colour",
                                 "colour_vi", "colour_nV")]


class Params(ct.Structure):
    _fields_ = [("SSA_RN_tol", F64), ("SSA_max_outer_loops", I32), ("SSA_max_residual_UV", F64),
                ("SSA_SOR_omega", F64), ("SSA_max_inner_loops", I32), ("m_enh_ssa", F64), ("m_enh_sia", F64),
                ("sliding_law", I32), ("beta_sq", F64), ("use_analytical_GL_flux", I32),
                ("zero_velocities", I32), ("nZ", I32), ("zeta", P), ("precision", I32),
                ("mixed_refold_sweeps", I32), ("fp64_exact", I32), ("mixed_fp32_viscosity", I32)]


SSA_IN_FIELDS = ("Hi", "Hb", "SL", "dHs_dx_shelf", "dHs_dy_shelf", "A_flow_mean", "mask_sheet", "Hi_Ac", "Hb_Ac",
                 "SL_Ac", "dHs_dx_shelf_Ac", "dHs_dy_shelf_Ac", "A_flow_mean_Ac", "beta_sq_AaAc", "mask_gl_Ac",
                 "dHi_dx_Ac", "dHi_dy_Ac", "dSL_dx_Ac", "dSL_dy_Ac", "dHb_dx_Ac", "dHb_dy_Ac")


class SsaIn(ct.Structure):
    _fields_ = [(n, P) for n in SSA_IN_FIELDS]


class SsaInout(ct.Structure):
    _fields_ = [(n, P) for n in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "N_AaAc")]


class SsaOut(ct.Structure):
    _fields_ = [(n, P) for n in ("Up_SSA_Ac", "Uo_SSA_Ac", "eta_AaAc", "S_AaAc", "tau_c_AaAc", "phi_fric_AaAc")]


class SsaStats(ct.Structure):
    _fields_ = [("status", I32), ("picard_iterations", I32), ("linear_solves", I32), ("resets", I32),
                ("not_converged", I32), ("total_sweeps", ct.c_int64), ("last_RN", F64),
                ("last_max_residual", F64), ("sweeps", I32 * 64), ("device_ms", F64)]


class SiaIn(ct.Structure):
    _fields_ = [(n, P) for n in ("mask_sheet_Ac", "Hi_Ac", "dHs_dx_Ac", "dHs_dy_Ac", "dHs_dp_Ac", "dHs_do_Ac",
                                 "A_flow_Ac")]


class SiaOut(ct.Structure):
    _fields_ = [(n, P) for n in ("D_SIA_3D_Ac", "D_SIA_Ac", "Ux_SIA_Ac", "Uy_SIA_Ac", "Up_SIA_Ac", "Uo_SIA_Ac",
                                 "U_SIA", "V_SIA", "D_SIA")]


MASK_NAMES = ("land", "ocean", "lake", "ice", "sheet", "shelf", "coast", "margin", "gl", "cf")
MASK_OUT_FIELDS = tuple("mask_" + n for n in MASK_NAMES) + ("mask",) + \
    tuple("mask_" + n + "_Ac" for n in MASK_NAMES) + ("mask_Ac",)


class MaskOut(ct.Structure):
    _fields_ = [(n, P) for n in MASK_OUT_FIELDS]


GEOM_MESH_FIELDS = ("nC", "C", "Nx", "Ny", "Aci", "Nx_Ac", "Ny_Ac", "No_Ac", "Np_Ac")


class GeometryMesh(ct.Structure):
    _fields_ = [(n, P) for n in GEOM_MESH_FIELDS]


GEOM_OUT_FIELDS = ("Hs", "dHi_dx", "dHi_dy", "dHs_dx", "dHs_dy", "dHs_dx_shelf", "dHs_dy_shelf",
                   "mask_ocean", "mask_ice", "mask_sheet", "mask_shelf", "Hi_Ac", "Hb_Ac", "SL_Ac", "Hs_Ac",
                   "dHi_dx_Ac", "dHi_dy_Ac", "dHi_dp_Ac", "dHi_do_Ac", "dHb_dx_Ac", "dHb_dy_Ac", "dHb_dp_Ac",
                   "dHb_do_Ac", "dHs_dx_Ac", "dHs_dy_Ac", "dHs_dp_Ac", "dHs_do_Ac", "dSL_dx_Ac", "dSL_dy_Ac",
                   "dSL_dp_Ac", "dSL_do_Ac", "dHs_dx_shelf_Ac", "dHs_dy_shelf_Ac", "mask_ocean_Ac", "mask_ice_Ac",
                   "mask_sheet_Ac", "mask_shelf_Ac", "mask_gl_Ac")


class GeometryOut(ct.Structure):
    _fields_ = [(n, P) for n in GEOM_OUT_FIELDS]


class Sia3dOut(ct.Structure):
    _fields_ = [(n, P) for n in ("U_3D", "V_3D", "W_3D")]


UFE_FLOW_ARRHENIUS, UFE_FLOW_EISMINT, UFE_FLOW_MISMIP_MOD = 0, 1, 2
PHYSPROP_OUT_FIELDS = ("A_flow", "Ti_pmp", "Cpi", "Ki", "A_flow_mean", "A_flow_Ac", "Ti_Ac", "A_flow_mean_Ac")


class PhyspropOut(ct.Structure):
    _fields_ = [(n, P) for n in PHYSPROP_OUT_FIELDS]


class TriangleMesh(ct.Structure):
    _fields_ = [("nTri", I32)] + [(n, P) for n in ("V", "R", "niTri", "iTri", "Tri", "NxTri", "NyTri")]


class ThicknessIn(ct.Structure):
    _fields_ = [(n, P) for n in ("A", "Cw", "Up_SIA_Ac", "Up_SSA_Ac", "SMB_year", "BMB", "mask_noice")] + \
               [("dt", F64), ("zero_edges", I32)]


class ThicknessOut(ct.Structure):
    _fields_ = [(n, P) for n in ("Hi_prev", "dHi_dt", "dVi_in")]


UFE_VJP_GMRES, UFE_VJP_SOR = 0, 1


class VjpParams(ct.Structure):
    _fields_ = [("tol", F64), ("max_sweeps", I32), ("omega", F64), ("method", I32), ("restart", I32),
                ("sweeps_per_iteration", I32)]


class VjpIn(ct.Structure):
    _fields_ = [(n, P) for n in ("dJ_dU", "dJ_dV", "dJ_dUx_Ac", "dJ_dUy_Ac")]


class VjpGeom(ct.Structure):
    _fields_ = [(n, P) for n in ("nC", "C", "Nx", "Ny", "Aci", "Nx_Ac", "Ny_Ac")]


VJP_OUT_FIELDS = ("dJ_dlogbeta_sq_AaAc", "dJ_dHi", "dJ_dhx_AaAc", "dJ_dhy_AaAc", "dJ_dHi_AaAc", "lambda_U_AaAc",
                  "lambda_V_AaAc", "dJ_dphi_fric_AaAc")


class VjpOut(ct.Structure):
    _fields_ = [(n, P) for n in VJP_OUT_FIELDS]


class VjpStats(ct.Structure):
    _fields_ = [("status", I32), ("sweeps", I32), ("last_rel_update", F64), ("device_ms", F64)]


class BatchConfig(ct.Structure):
    _fields_ = [("team_ctas", I32), ("rows_per_cta", I32), ("block", I32), ("use_graph", I32)]


class BatchPlan(ct.Structure):
    _fields_ = [("n_classes", I32), ("class_team_ctas", I32 * 16), ("class_teams", I32 * 16), ("grid_ctas", I32)]


class BatchTiming(ct.Structure):
    _fields_ = [("device_ms", F64), ("solve_ms", F64), ("member_p50_ms", F64), ("member_p99_ms", F64),
                ("member_max_ms", F64), ("member_ms", P), ("n_active", I32), ("n_teams", I32),
                ("n_classes", I32), ("grid_ctas", I32), ("max_team_ctas", I32), ("block", I32)]


class BatchTuneEntry(ct.Structure):
    _fields_ = [("rows_per_cta", I32), ("block", I32), ("grid_ctas", I32), ("n_classes", I32),
                ("device_ms", F64), ("member_p99_ms", F64)]


class BaseMeshC(ct.Structure):
    _fields_ = [("nV", I32), ("nTri", I32), ("nC_mem", I32)] + \
               [(n, P) for n in ("V", "nC", "C", "niTri", "iTri", "Tri", "edge_index")]


AAAC_FIELDS = ("Nx", "Ny", "Nxx", "Nxy", "Nyy", "iAci", "Aci", "VAc", "Nx_Ac", "Ny_Ac", "No_Ac", "Np_Ac",
               "edge_index_Ac", "VAaAc", "nCAaAc", "CAaAc", "Nx_AaAc", "Ny_AaAc", "Nxx_AaAc", "Nxy_AaAc",
               "Nyy_AaAc", "colour", "colour_vi", "colour_nV")


class AaAcMeshC(ct.Structure):
    _fields_ = [("nAc", I32), ("nVAaAc", I32)] + [(n, P) for n in AAAC_FIELDS]


# Every symbol include/ufemism_gb300.h declares, with its prototype.
PROTOTYPES = {
    "ufe_init": (I32, [ct.c_int]),
    "ufe_last_error_string": (ct.c_char_p, []),
    "ufe_mesh_create": (I32, [ct.POINTER(MeshDesc), ct.POINTER(P)]),
    "ufe_mesh_destroy": (I32, [P]),
    "ufe_mesh_stream": (P, [P]),
    "ufe_ssa_solve": (I32, [P, ct.POINTER(Params), ct.POINTER(SsaIn), ct.POINTER(SsaInout), ct.POINTER(SsaOut),
                            ct.POINTER(SsaStats)]),
    "ufe_ssa_upload": (I32, [P, ct.POINTER(Params), ct.POINTER(SsaIn), ct.POINTER(SsaInout)]),
    "ufe_ssa_run": (I32, [P, ct.POINTER(Params), ct.POINTER(SsaStats)]),
    "ufe_ssa_download": (I32, [P, ct.POINTER(SsaInout), ct.POINTER(SsaOut)]),
    "ufe_sia_solve": (I32, [P, ct.POINTER(Params), ct.POINTER(SiaIn), ct.POINTER(SiaOut)]),
    "ufe_ssa_frictional_heating": (I32, [P, P, P]),
    "ufe_sia_solve_noalloc": (I32, [P, ct.POINTER(Params), ct.POINTER(SiaIn), ct.POINTER(SiaOut)]),
    "ufe_geometry_attach": (I32, [P, ct.POINTER(GeometryMesh)]),
    "ufe_geometry_update": (I32, [P, P, P, P, ct.POINTER(GeometryOut)]),
    "ufe_geometry_masks": (I32, [P, ct.POINTER(MaskOut)]),
    "ufe_ssa_upload_geometry": (I32, [P, ct.POINTER(Params), P, P, P, P, P, P, ct.POINTER(SsaInout)]),
    "ufe_sia_solve_geometry": (I32, [P, ct.POINTER(Params), P, ct.POINTER(SiaOut)]),
    "ufe_sia3d_solve": (I32, [P, ct.POINTER(Params), P, P, ct.POINTER(Sia3dOut)]),
    "ufe_ice_physical_properties": (I32, [P, ct.POINTER(Params), I32, ct.c_double, P, ct.POINTER(PhyspropOut)]),
    "ufe_triangles_attach": (I32, [P, ct.POINTER(TriangleMesh)]),
    "ufe_upwind_derivatives_3d": (I32, [P, ct.POINTER(Params), P, P, P, P, P, ct.POINTER(ct.c_int64)]),
    "ufe_thickness_update": (I32, [P, ct.POINTER(ThicknessIn), P, ct.POINTER(ThicknessOut)]),
    "ufe_ssa_vjp": (I32, [P, ct.POINTER(Params), ct.POINTER(VjpParams), ct.POINTER(VjpIn), ct.POINTER(VjpGeom),
                          ct.POINTER(VjpOut), ct.POINTER(VjpStats)]),
    "ufe_batch_plan": (I32, [ct.POINTER(I32), I32, ct.POINTER(BatchConfig), I32, ct.POINTER(I32),
                             ct.POINTER(BatchPlan)]),
    "ufe_ssa_solve_batched": (I32, [I32, ct.POINTER(MeshDesc), ct.POINTER(BatchConfig), ct.POINTER(Params),
                                    ct.POINTER(SsaIn), ct.POINTER(SsaInout), ct.POINTER(SsaOut),
                                    ct.POINTER(SsaStats)]),
    "ufe_batch_autotune": (I32, [I32, ct.POINTER(MeshDesc), ct.POINTER(Params), ct.POINTER(SsaIn),
                                 ct.POINTER(SsaInout), ct.POINTER(BatchConfig), ct.POINTER(BatchTuneEntry), I32,
                                 ct.POINTER(I32)]),
    "ufe_batch_create": (I32, [ct.POINTER(MeshDesc), I32, ct.POINTER(BatchConfig), ct.POINTER(P)]),
    "ufe_batch_destroy": (I32, [P]),
    "ufe_batch_upload": (I32, [P, I32, ct.POINTER(Params), ct.POINTER(SsaIn), ct.POINTER(SsaInout)]),
    "ufe_batch_run": (I32, [P, ct.POINTER(Params), ct.POINTER(SsaStats), ct.POINTER(BatchTiming)]),
    "ufe_batch_download": (I32, [P, I32, ct.POINTER(SsaInout), ct.POINTER(SsaOut)]),
    "ufe_aaac_build": (I32, [ct.POINTER(BaseMeshC), ct.POINTER(AaAcMeshC)]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the native library (building it first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("libufemism_gb300.so is not built; run ufemism_gb300.build.build()")
    L = ct.CDLL(_build.LIB)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return load().ufe_last_error_string().decode(errors="replace")


class UfeError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__("%s failed: %s (%d): %s" % (where, STATUS_NAMES.get(status, "?"), status, last_error()))
