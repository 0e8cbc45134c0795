"""ctypes binding of the CPU oracle (ufe_oracle.h) -- TEST INFRASTRUCTURE ONLY.

Used by the tests, by ``__graft_entry__.smoke()`` as the checker, and by the CPU-baseline
leg of ``bench.py``. Never part of the product path.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libufe_oracle.so")
_lib = None

OR_OK, OR_NOT_CONVERGED, OR_RESET_ONCE = 0, 1, 2
OR_ERR_DIVERGED, OR_ERR_BAD_MESH, OR_ERR_COLOUR_IDENTIFY = -1, -2, -3
OR_ERR_COLOUR_STUCK, OR_ERR_COLOUR_QUEUE, OR_ERR_COLOUR_INVALID = -4, -5, -6

ZETA_DEFAULT = np.array([0.00, 0.10, 0.20, 0.30, 0.40, 0.50, 0.60, 0.70, 0.80, 0.90,
                         0.925, 0.95, 0.975, 0.99, 1.00])  # configuration_module.f90:124-126


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB) or any(
            os.path.getmtime(os.path.join(_HERE, f)) > os.path.getmtime(_LIB)
            for f in ("ufe_oracle_mesh.c", "ufe_oracle_solve.c", "ufe_oracle_thickness.c", "ufe_oracle_sia3d.c",
                      "ufe_oracle_physprop.c", "ufe_oracle_upwind.c", "ufe_oracle_masks.c", "ufe_oracle.h")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ct.CDLL(_LIB)
    return _lib


P = ct.c_void_p
I32 = ct.c_int32


class _Base(ct.Structure):
    _fields_ = [("nV", I32), ("nTri", I32), ("nC_mem", I32),
                ("V", P), ("nC", P), ("C", P), ("niTri", P), ("iTri", P), ("Tri", P),
                ("edge_index", P)]


class _AaAc(ct.Structure):
    _fields_ = [("nAc", I32), ("nVAaAc", I32),
                ("Nx", P), ("Ny", P), ("Nxx", P), ("Nxy", P), ("Nyy", P),
                ("iAci", P), ("Aci", P), ("VAc", P), ("Nx_Ac", P), ("Ny_Ac", P), ("No_Ac", P),
                ("Np_Ac", P), ("edge_index_Ac", P), ("VAaAc", P), ("nCAaAc", P), ("CAaAc", P),
                ("Nx_AaAc", P), ("Ny_AaAc", P), ("Nxx_AaAc", P), ("Nxy_AaAc", P), ("Nyy_AaAc", P),
                ("colour", P), ("colour_vi", P), ("colour_nV", P)]


class _Params(ct.Structure):
    _fields_ = [("SSA_RN_tol", ct.c_double), ("SSA_max_outer_loops", I32),
                ("SSA_max_residual_UV", ct.c_double), ("SSA_SOR_omega", ct.c_double),
                ("SSA_max_inner_loops", I32), ("m_enh_ssa", ct.c_double), ("m_enh_sia", ct.c_double),
                ("sliding_law", I32), ("use_analytical_GL_flux", I32), ("zero_velocities", I32),
                ("nZ", I32), ("zeta", P), ("n_threads", I32), ("replay_picard", I32),
                ("replay_sweeps", P), ("progress", P)]


class _SSA(ct.Structure):
    _fields_ = [(n, P) for n in ("Hi", "Hb", "SL", "dHs_dx_shelf", "dHs_dy_shelf", "A_flow_mean",
                                 "mask_sheet", "Hi_Ac", "Hb_Ac", "SL_Ac", "dHs_dx_shelf_Ac",
                                 "dHs_dy_shelf_Ac", "A_flow_mean_Ac", "beta_sq_AaAc")] + \
               [("beta_sq_const", ct.c_double)] + \
               [(n, P) for n in ("mask_gl_Ac", "dHi_dx_Ac", "dHi_dy_Ac", "dSL_dx_Ac", "dSL_dy_Ac",
                                 "dHb_dx_Ac", "dHb_dy_Ac", "U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac",
                                 "N_AaAc", "Up_SSA_Ac", "Uo_SSA_Ac", "eta_AaAc", "S_AaAc",
                                 "tau_c_AaAc", "phi_fric_AaAc")]


class _Stats(ct.Structure):
    _fields_ = [("picard_iterations", I32), ("linear_solves", I32), ("total_sweeps", ct.c_int64),
                ("resets", I32), ("not_converged", I32), ("last_RN", ct.c_double),
                ("last_max_residual", ct.c_double), ("sweeps", I32 * 64)]


class _SIA(ct.Structure):
    _fields_ = [(n, P) for n in ("mask_sheet_Ac", "Hi_Ac", "dHs_dx_Ac", "dHs_dy_Ac", "dHs_dp_Ac",
                                 "dHs_do_Ac", "A_flow_Ac", "D_SIA_3D_Ac", "D_SIA_Ac", "Ux_SIA_Ac",
                                 "Uy_SIA_Ac", "Up_SIA_Ac", "Uo_SIA_Ac", "U_SIA", "V_SIA", "D_SIA")]


_GEOM_IN = ("Hi", "Hb", "SL")
_GEOM_AA_D = ("Hs", "dHi_dx", "dHi_dy", "dHs_dx", "dHs_dy", "dHs_dx_shelf", "dHs_dy_shelf")
_GEOM_AA_I = ("mask_ocean", "mask_ice", "mask_sheet", "mask_shelf")
_GEOM_AC_D = ("Hi_Ac", "Hb_Ac", "SL_Ac", "Hs_Ac",
              "dHi_dx_Ac", "dHi_dy_Ac", "dHi_dp_Ac", "dHi_do_Ac",
              "dHb_dx_Ac", "dHb_dy_Ac", "dHb_dp_Ac", "dHb_do_Ac",
              "dHs_dx_Ac", "dHs_dy_Ac", "dHs_dp_Ac", "dHs_do_Ac",
              "dSL_dx_Ac", "dSL_dy_Ac", "dSL_dp_Ac", "dSL_do_Ac",
              "dHs_dx_shelf_Ac", "dHs_dy_shelf_Ac")
_GEOM_AC_I = ("mask_ocean_Ac", "mask_ice_Ac", "mask_sheet_Ac", "mask_shelf_Ac", "mask_gl_Ac")


class _Geom(ct.Structure):
    _fields_ = [(n, P) for n in _GEOM_IN + _GEOM_AA_D + _GEOM_AA_I + _GEOM_AC_D + _GEOM_AC_I]


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def _i32(a):
    return np.asfortranarray(a, dtype=np.int32)


@dataclass
class AaAcMesh:
    """Base mesh plus everything make_Ac_mesh / get_neighbour_functions / the five-colouring
    produce, in the reference's layout (1-based index values, Fortran-order arrays)."""
    base: object
    nAc: int
    nVAaAc: int
    arrays: dict = field(default_factory=dict)
    colour_status: int = 0
    reduce_iterations: int = 0

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays", {})
        if name in arrays:
            return arrays[name]
        raise AttributeError(name)


def _base_struct(base):
    keep = dict(V=_f64(base.V), nC=_i32(base.nC), C=_i32(base.C), niTri=_i32(base.niTri),
                iTri=_i32(base.iTri), Tri=_i32(base.Tri), edge_index=_i32(base.edge_index))
    s = _Base(base.nV, base.nTri, keep["C"].shape[1], *(_ptr(keep[k]) for k in
                                                         ("V", "nC", "C", "niTri", "iTri", "Tri", "edge_index")))
    return s, keep


def _aaac_struct(m: AaAcMesh):
    a = m.arrays
    return _AaAc(m.nAc, m.nVAaAc, *(_ptr(a[k]) for k in (
        "Nx", "Ny", "Nxx", "Nxy", "Nyy", "iAci", "Aci", "VAc", "Nx_Ac", "Ny_Ac", "No_Ac", "Np_Ac",
        "edge_index_Ac", "VAaAc", "nCAaAc", "CAaAc", "Nx_AaAc", "Ny_AaAc", "Nxx_AaAc", "Nxy_AaAc",
        "Nyy_AaAc", "colour", "colour_vi", "colour_nV")))


def build_aaac(base, colour: bool = True) -> AaAcMesh:
    """make_Ac_mesh + get_neighbour_functions + calculate_five_colouring_AaAc."""
    L = lib()
    nV, nTri, nCm = base.nV, base.nTri, base.C.shape[1]
    nAc = nV + nTri - 1
    nA = nV + nAc
    z = lambda *s: np.zeros(s, dtype=np.float64, order="F")
    zi = lambda *s: np.zeros(s, dtype=np.int32, order="F")
    arr = dict(Nx=z(nV, nCm + 1), Ny=z(nV, nCm + 1), Nxx=z(nV, nCm + 1), Nxy=z(nV, nCm + 1),
               Nyy=z(nV, nCm + 1), iAci=zi(nV, nCm), Aci=zi(nAc, 4), VAc=z(nAc, 2),
               Nx_Ac=z(nAc, 4), Ny_Ac=z(nAc, 4), No_Ac=z(nAc, 4), Np_Ac=z(nAc),
               edge_index_Ac=zi(nAc), VAaAc=z(nA, 2), nCAaAc=zi(nA), CAaAc=zi(nA, nCm),
               Nx_AaAc=z(nA, nCm + 1), Ny_AaAc=z(nA, nCm + 1), Nxx_AaAc=z(nA, nCm + 1),
               Nxy_AaAc=z(nA, nCm + 1), Nyy_AaAc=z(nA, nCm + 1), colour=zi(nA),
               colour_vi=zi(nA, 5), colour_nV=zi(5))
    m = AaAcMesh(base=base, nAc=nAc, nVAaAc=nA, arrays=arr)
    bs, keep = _base_struct(base)
    ms = _aaac_struct(m)
    rc = L.or_build_aaac(ct.byref(bs), ct.byref(ms))
    if rc != OR_OK:
        raise RuntimeError("or_build_aaac failed: %d" % rc)
    if colour:
        it = I32(0)
        m.colour_status = L.or_five_colouring(ct.byref(bs), ct.byref(ms), ct.byref(it))
        m.reduce_iterations = it.value
    return m


def _vp(a):
    return ct.c_void_p(a.ctypes.data)


def neighbour_functions_vertex(V_vi, V_vc, is_edge):
    n = V_vc.shape[0]
    vc = _f64(V_vc)
    vi = _f64(np.asarray(V_vi))
    out = [np.zeros(n + 1) for _ in range(5)]
    lib().or_neighbour_functions_vertex(_vp(vi), ct.c_int(n), _vp(vc), ct.c_int(n), ct.c_int(int(is_edge)),
                                        *(_vp(o) for o in out))
    return out


def default_params(**kw):
    """Solver knobs as used on the benchmark workloads (Picard tol 1e-3, SOR omega 1.3,
    SOR tol 1e-4 m/yr, m_enh = 1, linear sliding), overridable by keyword."""
    p = dict(SSA_RN_tol=1e-3, SSA_max_outer_loops=50, SSA_max_residual_UV=1e-4, SSA_SOR_omega=1.3,
             SSA_max_inner_loops=10000, m_enh_ssa=1.0, m_enh_sia=1.0, sliding_law=1,
             use_analytical_GL_flux=0, zero_velocities=0, zeta=ZETA_DEFAULT, n_threads=1,
             replay_picard=0, replay_sweeps=None, progress=None)
    p.update(kw)
    return p


def _params_struct(p):
    zeta = _f64(p["zeta"])
    rs = None if p.get("replay_sweeps") is None else np.ascontiguousarray(p["replay_sweeps"], dtype=np.int32)
    s = _Params(p["SSA_RN_tol"], p["SSA_max_outer_loops"], p["SSA_max_residual_UV"], p["SSA_SOR_omega"],
                p["SSA_max_inner_loops"], p["m_enh_ssa"], p["m_enh_sia"], p["sliding_law"],
                p["use_analytical_GL_flux"], p["zero_velocities"], zeta.size, _ptr(zeta),
                p["n_threads"], p["replay_picard"], _ptr(rs), _ptr(p.get("progress")))
    return s, (zeta, rs)


def update_geometry(m: AaAcMesh, Hi, Hb, SL) -> dict:
    """Geometry part of update_general_ice_model_data: Ac maps, Hs, masks, slopes."""
    nV, nAc = m.base.nV, m.nAc
    g = {"Hi": _f64(Hi), "Hb": _f64(Hb), "SL": _f64(SL)}
    for k in _GEOM_AA_D:
        g[k] = np.zeros(nV)
    for k in _GEOM_AA_I:
        g[k] = np.zeros(nV, dtype=np.int32)
    for k in _GEOM_AC_D:
        g[k] = np.zeros(nAc)
    for k in _GEOM_AC_I:
        g[k] = np.zeros(nAc, dtype=np.int32)
    gs = _Geom(*(_ptr(g[k]) for k in _GEOM_IN + _GEOM_AA_D + _GEOM_AA_I + _GEOM_AC_D + _GEOM_AC_I))
    bs, keep = _base_struct(m.base)
    ms = _aaac_struct(m)
    rc = lib().or_update_geometry(ct.byref(bs), ct.byref(ms), ct.byref(gs))
    if rc != OR_OK:
        raise RuntimeError("or_update_geometry failed: %d" % rc)
    return g


def solve_ssa(m: AaAcMesh, fields: dict, params: dict):
    """solve_SSA. ``fields`` holds the inputs (see or_ssa_fields) and optional warm-start
    U_SSA/V_SSA/Ux_SSA_Ac/Uy_SSA_Ac/N_AaAc. Returns (rc, outputs dict, stats dict)."""
    nV, nAc, nA = m.base.nV, m.nAc, m.nVAaAc
    f = dict(fields)
    out = {}
    for k, n in (("U_SSA", nV), ("V_SSA", nV), ("Ux_SSA_Ac", nAc), ("Uy_SSA_Ac", nAc), ("N_AaAc", nA)):
        out[k] = np.array(f.get(k, np.zeros(n)), dtype=np.float64, copy=True)
    for k, n in (("Up_SSA_Ac", nAc), ("Uo_SSA_Ac", nAc), ("eta_AaAc", nA), ("S_AaAc", nA),
                 ("tau_c_AaAc", nA), ("phi_fric_AaAc", nA)):
        out[k] = np.zeros(n)
    keep = {}

    def g(k, dt=np.float64):
        v = f.get(k)
        if v is None:
            return None
        a = np.ascontiguousarray(v, dtype=dt)
        keep[k] = a
        return _ptr(a)

    beta = f.get("beta_sq_AaAc")
    s = _SSA(g("Hi"), g("Hb"), g("SL"), g("dHs_dx_shelf"), g("dHs_dy_shelf"), g("A_flow_mean"),
             g("mask_sheet", np.int32), g("Hi_Ac"), g("Hb_Ac"), g("SL_Ac"), g("dHs_dx_shelf_Ac"),
             g("dHs_dy_shelf_Ac"), g("A_flow_mean_Ac"), g("beta_sq_AaAc"),
             float(f.get("beta_sq_const", 1e3)) if beta is None else 0.0,
             g("mask_gl_Ac", np.int32), g("dHi_dx_Ac"), g("dHi_dy_Ac"), g("dSL_dx_Ac"), g("dSL_dy_Ac"),
             g("dHb_dx_Ac"), g("dHb_dy_Ac"),
             *(_ptr(out[k]) for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "N_AaAc", "Up_SSA_Ac",
                                      "Uo_SSA_Ac", "eta_AaAc", "S_AaAc", "tau_c_AaAc", "phi_fric_AaAc")))
    st = _Stats()
    ps, pkeep = _params_struct(params)
    bs, bkeep = _base_struct(m.base)
    ms = _aaac_struct(m)
    rc = lib().or_solve_SSA(ct.byref(bs), ct.byref(ms), ct.byref(ps), ct.byref(s), ct.byref(st))
    stats = dict(picard_iterations=st.picard_iterations, linear_solves=st.linear_solves,
                 total_sweeps=st.total_sweeps, resets=st.resets, not_converged=st.not_converged,
                 last_RN=st.last_RN, last_max_residual=st.last_max_residual,
                 sweeps=list(st.sweeps)[:min(64, st.linear_solves)])
    return rc, out, stats


def solve_sia(m: AaAcMesh, fields: dict, params: dict):
    nV, nAc = m.base.nV, m.nAc
    nZ = len(params["zeta"])
    out = dict(D_SIA_3D_Ac=np.zeros((nAc, nZ), order="F"), D_SIA_Ac=np.zeros(nAc), Ux_SIA_Ac=np.zeros(nAc),
               Uy_SIA_Ac=np.zeros(nAc), Up_SIA_Ac=np.zeros(nAc), Uo_SIA_Ac=np.zeros(nAc),
               U_SIA=np.zeros(nV), V_SIA=np.zeros(nV), D_SIA=np.zeros(nV))
    keep = dict(mask_sheet_Ac=_i32(fields["mask_sheet_Ac"]), Hi_Ac=_f64(fields["Hi_Ac"]),
                dHs_dx_Ac=_f64(fields["dHs_dx_Ac"]), dHs_dy_Ac=_f64(fields["dHs_dy_Ac"]),
                dHs_dp_Ac=_f64(fields["dHs_dp_Ac"]), dHs_do_Ac=_f64(fields["dHs_do_Ac"]),
                A_flow_Ac=_f64(fields["A_flow_Ac"]))
    s = _SIA(*(_ptr(keep[k]) for k in ("mask_sheet_Ac", "Hi_Ac", "dHs_dx_Ac", "dHs_dy_Ac", "dHs_dp_Ac",
                                       "dHs_do_Ac", "A_flow_Ac")),
             *(_ptr(out[k]) for k in ("D_SIA_3D_Ac", "D_SIA_Ac", "Ux_SIA_Ac", "Uy_SIA_Ac", "Up_SIA_Ac",
                                      "Uo_SIA_Ac", "U_SIA", "V_SIA", "D_SIA")))
    ps, pkeep = _params_struct(params)
    bs, bkeep = _base_struct(m.base)
    ms = _aaac_struct(m)
    rc = lib().or_solve_SIA(ct.byref(bs), ct.byref(ms), ct.byref(ps), ct.byref(s))
    if rc != OR_OK:
        raise RuntimeError("or_solve_SIA failed: %d" % rc)
    return out


def neumann(m: AaAcMesh, d):
    a = np.array(d, dtype=np.float64, copy=True)
    bs, keep = _base_struct(m.base)
    ms = _aaac_struct(m)
    lib().or_neumann_AaAc(ct.byref(bs), ct.byref(ms), _vp(a))
    return a


def ddx_ddy_aaac(m: AaAcMesh, d):
    d = np.ascontiguousarray(d, dtype=np.float64)
    dx = np.zeros(m.nVAaAc)
    dy = np.zeros(m.nVAaAc)
    ms = _aaac_struct(m)
    lib().or_ddx_ddy_AaAc(ct.byref(ms), ct.c_int(m.base.C.shape[1]), _vp(d), _vp(dx), _vp(dy))
    return dx, dy


def thickness_change(m: AaAcMesh, A, Cw, Up_SIA_Ac, Up_SSA_Ac, SMB_year, BMB, dt, Hi, mask_noice=None,
                     zero_edges=True):
    """calculate_ice_thickness_change. Returns (Hi_new, Hi_prev, dHi_dt, dVi_in)."""
    base = m.base
    nV = base.nV
    ncm = base.C.shape[1]
    Hi_new = np.array(Hi, dtype=np.float64, copy=True)
    Hi_prev = np.zeros(nV)
    dHi_dt = np.zeros(nV)
    dVi_in = np.zeros((nV, ncm), order="F")
    keep = [_f64(A), _f64(Cw), _f64(Up_SIA_Ac), _f64(Up_SSA_Ac), _f64(SMB_year), _f64(BMB)]
    mk = None if mask_noice is None else _i32(mask_noice)
    bs, bkeep = _base_struct(base)
    ms = _aaac_struct(m)
    rc = lib().or_thickness_change(ct.byref(bs), ct.byref(ms), *(_vp(k) for k in keep), None if mk is None else _vp(mk),
                                   ct.c_double(dt), ct.c_int(1 if zero_edges else 0), _vp(Hi_new), _vp(Hi_prev),
                                   _vp(dHi_dt), _vp(dVi_in))
    if rc != OR_OK:
        raise RuntimeError("or_thickness_change failed: %d" % rc)
    return Hi_new, Hi_prev, dHi_dt, dVi_in


def frictional_heating(mask_sheet, tau_c_AaAc, U, V):
    """bottom_frictional_heating on the Aa vertices (U, V, mask_sheet of length nV)."""
    nV = len(U)
    out = np.zeros(nV)
    keep = [_i32(mask_sheet), _f64(tau_c_AaAc), _f64(U), _f64(V)]
    lib().or_frictional_heating(ct.c_int(nV), *(_vp(k) for k in keep), _vp(out))
    return out


def solve_sia_3d(m: AaAcMesh, g: dict, A_flow, dHb_dt, U_SSA, V_SSA, zeta=None, m_enh_sia=1.0):
    """solve_SIA_3D with the geometry fields of update_geometry. Returns (U_3D, V_3D, W_3D),
    each (nV, nZ)."""
    base = m.base
    nV = base.nV
    z = np.ascontiguousarray(ZETA_DEFAULT if zeta is None else zeta, dtype=np.float64)
    nZ = z.size
    outs = [np.zeros((nV, nZ), order="F") for _ in range(3)]
    keep = [_f64(g["Hi"]), _i32(g["mask_shelf"]), _i32(g["mask_sheet"]), _f64(g["dHs_dx"]), _f64(g["dHs_dy"]),
            _f64(g["dHi_dx"]), _f64(g["dHi_dy"]), _f64(A_flow), _f64(dHb_dt), _f64(U_SSA), _f64(V_SSA)]
    bs, bkeep = _base_struct(base)
    ms = _aaac_struct(m)
    rc = lib().or_solve_SIA_3D(ct.byref(bs), ct.byref(ms), _vp(z), ct.c_int(nZ), ct.c_double(m_enh_sia),
                               *(_vp(k) for k in keep), *(_vp(o) for o in outs))
    if rc != OR_OK:
        raise RuntimeError("or_solve_SIA_3D failed: %d" % rc)
    return tuple(outs)


def ice_physical_properties(m: AaAcMesh, Hi, mask_sheet, mask_sheet_Ac, Ti=None, flow_law=0, time=0.0, zeta=None):
    """ice_physical_properties (flow_law 0: Arrhenius from Ti, 1: EISMINT-type constants,
    2: MISMIP_mod). Returns a dict of A_flow, Ti_pmp, Cpi, Ki (nV, nZ), A_flow_mean (nV),
    A_flow_Ac, Ti_Ac (nAc, nZ), A_flow_mean_Ac (nAc); the fields a law does not write stay NaN."""
    nV, nAc = m.base.nV, m.nAc
    z = np.ascontiguousarray(ZETA_DEFAULT if zeta is None else zeta, dtype=np.float64)
    nZ = z.size
    out = {k: np.full((nV, nZ), np.nan, order="F") for k in ("A_flow", "Ti_pmp", "Cpi", "Ki")}
    out.update(A_flow_Ac=np.full((nAc, nZ), np.nan, order="F"), Ti_Ac=np.full((nAc, nZ), np.nan, order="F"),
               A_flow_mean=np.full(nV, np.nan), A_flow_mean_Ac=np.full(nAc, np.nan))
    keep = [_f64(Hi), _i32(mask_sheet), _i32(mask_sheet_Ac), None if Ti is None else _f64(Ti), _i32(m.Aci)]
    rc = lib().or_ice_physical_properties(
        ct.c_int(nV), ct.c_int(nAc), ct.c_int(nZ), _vp(z), _vp(keep[4]), ct.c_int(flow_law), ct.c_double(time),
        _vp(keep[0]), _vp(keep[1]), _vp(keep[2]), None if keep[3] is None else _vp(keep[3]),
        *(_vp(out[k]) for k in ("A_flow", "A_flow_Ac", "A_flow_mean", "A_flow_mean_Ac", "Ti_pmp", "Cpi", "Ki",
                                "Ti_Ac")))
    if rc != OR_OK:
        raise RuntimeError("or_ice_physical_properties failed: %d" % rc)
    return out


def triangle_functions(base):
    """NxTri, NyTri (nTri, 3) of get_neighbour_functions."""
    NxT = np.zeros((base.nTri, 3), order="F")
    NyT = np.zeros((base.nTri, 3), order="F")
    bs, bkeep = _base_struct(base)
    lib().or_triangle_functions(ct.byref(bs), _vp(NxT), _vp(NyT))
    return NxT, NyT


def vertex_resolution(base, domain_width=None):
    """mesh%R: the distance from each vertex to its nearest neighbour."""
    V = np.asarray(base.V)
    w = float(V[:, 0].max() - V[:, 0].min()) if domain_width is None else float(domain_width)
    R = np.zeros(base.nV)
    bs, bkeep = _base_struct(base)
    lib().or_vertex_resolution(ct.byref(bs), ct.c_double(w), _vp(R))
    return R


def upwind_derivatives_3d(m: AaAcMesh, R, NxTri, NyTri, U, V, d):
    """get_upwind_derivative_vertex_3D for every vertex and layer. Returns (ddx, ddy,
    number of pairs without an upwind triangle)."""
    base = m.base
    keep = [_f64(R), _f64(NxTri), _f64(NyTri), _f64(U), _f64(V), _f64(d)]
    nV, nZ = keep[3].shape
    ddx = np.zeros((nV, nZ), order="F")
    ddy = np.zeros((nV, nZ), order="F")
    bs, bkeep = _base_struct(base)
    ms = _aaac_struct(m)
    f = lib().or_upwind_derivatives_3d
    f.restype = ct.c_longlong
    missing = f(ct.byref(bs), ct.byref(ms), ct.c_int(nZ), *(_vp(k) for k in keep), _vp(ddx), _vp(ddy))
    return ddx, ddy, int(missing)


MASK_NAMES = ("land", "ocean", "lake", "ice", "sheet", "shelf", "coast", "margin", "gl", "cf", "type")


def determine_masks(m: AaAcMesh, Hi, Hb, SL) -> dict:
    """determine_masks in full: mask_<name> (nV) and mask_<name>_Ac (nAc) for every name of
    MASK_NAMES, "type" being the combined type mask."""
    base = m.base
    nV, nAc = base.nV, m.nAc
    keep = [_f64(Hi), _f64(Hb), _f64(SL)]
    ac_in = [np.zeros(nAc) for _ in range(3)]
    for a, o in zip(keep, ac_in):
        lib().or_map_Aa_to_Ac(ct.byref(_aaac_struct(m)), ct.c_int(nV), _vp(a), _vp(o))
    aa = np.zeros((nV, len(MASK_NAMES)), dtype=np.int32, order="F")
    ac = np.zeros((nAc, len(MASK_NAMES)), dtype=np.int32, order="F")
    bs, bkeep = _base_struct(base)
    ms = _aaac_struct(m)
    lib().or_determine_masks(ct.byref(bs), ct.byref(ms), *(_vp(a) for a in keep), *(_vp(a) for a in ac_in),
                             _vp(aa), _vp(ac))
    out = {}
    for k, name in enumerate(MASK_NAMES):
        out["mask_" + name] = aa[:, k].copy()
        out["mask_" + name + "_Ac"] = ac[:, k].copy()
    return out
