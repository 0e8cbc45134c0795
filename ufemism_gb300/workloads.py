"""Seeded synthetic inputs for the ice-velocity solve.

The reference's benchmark geometries are hard-coded formulas (reference_fields_module.f90),
not datasets; these generators build the geometries the benchmark workloads are quoted on:

* Vialov dome H(r) = H0 (1 - (r/R)^(4/3))^(3/8), R = 750 km, flat bed at 0 m, grounded;
* marine variant: bed sloping from +500 m at the centre to -1000 m at r = 750 km plus a
  seeded Gaussian random field (sigma 50 m, correlation length 40 km), sea level 0 m, so
  the thin margin floats (is_floating, general_ice_model_data_module.f90:464-475);
* log-normal friction fields log(beta^2) = GRF(mean ln 1e3, std, correlation length).

``prepare_inputs`` is the geometry part of update_general_ice_model_data
(general_ice_model_data_module.f90:23-96): Ac maps, surface height, masks, Aa and Ac slopes
and the shelf-slope rule, vectorised with numpy for input generation.
"""
from __future__ import annotations

import numpy as np

ICE_DENSITY = 910.0
SEAWATER_DENSITY = 1028.0
A_FLOW = 1e-16  # Pa^-3 yr^-1


def grf(x, y, sigma, ell, seed, modes=256):
    """Stationary Gaussian random field with covariance sigma^2 exp(-r^2 / (2 ell^2)),
    by random Fourier features (a seeded spectral synthesis)."""
    rng = np.random.default_rng(seed)
    k = rng.normal(0.0, 1.0 / ell, size=(modes, 2))
    ph = rng.uniform(0.0, 2 * np.pi, size=modes)
    out = np.zeros(np.shape(x))
    for c in range(0, modes, 32):
        arg = np.outer(x, k[c:c + 32, 0]) + np.outer(y, k[c:c + 32, 1]) + ph[c:c + 32]
        out += np.cos(arg).sum(axis=1)
    return sigma * np.sqrt(2.0 / modes) * out


def dome_thickness(x, y, H0=3600.0, R=750e3):
    r = np.hypot(x, y)
    s = np.clip(1.0 - (r / R) ** (4.0 / 3.0), 0.0, None)
    return np.where(r < R, H0 * s ** (3.0 / 8.0), 0.0)


def dome_geometry(base, H0=3600.0, R=750e3):
    x, y = base.V[:, 0], base.V[:, 1]
    return dome_thickness(x, y, H0, R), np.zeros(base.nV), np.zeros(base.nV)


def marine_geometry(base, seed=20261206, H0=3600.0, R=750e3):
    x, y = base.V[:, 0], base.V[:, 1]
    r = np.hypot(x, y)
    Hb = 500.0 - 1500.0 * (r / R) + grf(x, y, 50.0, 40e3, seed)
    return dome_thickness(x, y, H0, R), Hb, np.zeros(base.nV)


def log_beta_field(mesh, std=1.0, ell=100e3, seed=20261207, mean=np.log(1e3)):
    xy = np.asarray(mesh.VAaAc)
    return mean + grf(xy[:, 0], xy[:, 1], std, ell, seed)


def _is_floating(Hi, Hb, SL):
    return Hi < ((SL - Hb) * SEAWATER_DENSITY) / ICE_DENSITY


def _ddx_ddy_aa(mesh, d):
    base = mesh.base
    nC = base.nC
    C = base.C - 1
    rows = np.arange(base.nV)
    Nx, Ny = np.asarray(mesh.Nx), np.asarray(mesh.Ny)
    dx = Nx[rows, nC] * d
    dy = Ny[rows, nC] * d
    for c in range(C.shape[1]):
        m = c < nC
        j = np.where(m, C[:, c], 0)
        dx = dx + np.where(m, Nx[:, c] * d[j], 0.0)
        dy = dy + np.where(m, Ny[:, c] * d[j], 0.0)
    return dx, dy


def _derivs_ac(mesh, d):
    Aci = np.asarray(mesh.Aci) - 1
    dx = np.zeros(mesh.nAc)
    dy = np.zeros(mesh.nAc)
    do = np.zeros(mesh.nAc)
    for n in range(4):
        dv = d[Aci[:, n]]
        dx = dx + mesh.Nx_Ac[:, n] * dv
        dy = dy + mesh.Ny_Ac[:, n] * dv
        do = do + mesh.No_Ac[:, n] * dv
    dp = mesh.Np_Ac * (d[Aci[:, 1]] - d[Aci[:, 0]])
    return dx, dy, dp, do


def prepare_inputs(mesh, Hi, Hb, SL, A=A_FLOW, nZ=15):
    """Fields solve_SSA and solve_SIA read, from Hi, Hb, SL on the Aa mesh."""
    Aci = np.asarray(mesh.Aci) - 1
    vi, vj = Aci[:, 0], Aci[:, 1]
    to_ac = lambda d: (d[vi] + d[vj]) / 2.0
    Hi_Ac, Hb_Ac, SL_Ac = to_ac(Hi), to_ac(Hb), to_ac(SL)
    rr = ICE_DENSITY / SEAWATER_DENSITY
    Hs = Hi + np.maximum(SL - rr * Hi, Hb)
    Hs_Ac = Hi_Ac + np.maximum(SL_Ac - rr * Hi_Ac, Hb_Ac)
    ocean = _is_floating(Hi, Hb, SL)
    ice = Hi > 0.0
    ocean_Ac = _is_floating(Hi_Ac, Hb_Ac, SL_Ac)
    ice_Ac = Hi_Ac > 0.0
    sheet, shelf = ice & ~ocean, ice & ocean
    sheet_Ac = ice_Ac & ~ocean_Ac
    gl_Ac = (sheet[vi] & shelf[vj]) | (sheet[vj] & shelf[vi])
    dHi_dx, dHi_dy = _ddx_ddy_aa(mesh, Hi)
    dHs_dx, dHs_dy = _ddx_ddy_aa(mesh, Hs)
    dHi_dx_Ac, dHi_dy_Ac, _, _ = _derivs_ac(mesh, Hi)
    dHb_dx_Ac, dHb_dy_Ac, _, _ = _derivs_ac(mesh, Hb)
    dHs_dx_Ac, dHs_dy_Ac, dHs_dp_Ac, dHs_do_Ac = _derivs_ac(mesh, Hs)
    dSL_dx_Ac, dSL_dy_Ac, _, _ = _derivs_ac(mesh, SL)
    shelf_f = 1.0 - rr
    ssa = dict(
        Hi=Hi, Hb=Hb, SL=SL,
        dHs_dx_shelf=np.where(ocean, shelf_f * dHi_dx, dHs_dx),
        dHs_dy_shelf=np.where(ocean, shelf_f * dHi_dy, dHs_dy),
        A_flow_mean=np.full(mesh.base.nV, A), mask_sheet=sheet.astype(np.int32),
        Hi_Ac=Hi_Ac, Hb_Ac=Hb_Ac, SL_Ac=SL_Ac,
        dHs_dx_shelf_Ac=np.where(ocean_Ac, shelf_f * dHi_dx_Ac, dHs_dx_Ac),
        dHs_dy_shelf_Ac=np.where(ocean_Ac, shelf_f * dHi_dy_Ac, dHs_dy_Ac),
        A_flow_mean_Ac=np.full(mesh.nAc, A),
        mask_gl_Ac=gl_Ac.astype(np.int32),
        dHi_dx_Ac=dHi_dx_Ac, dHi_dy_Ac=dHi_dy_Ac, dSL_dx_Ac=dSL_dx_Ac, dSL_dy_Ac=dSL_dy_Ac,
        dHb_dx_Ac=dHb_dx_Ac, dHb_dy_Ac=dHb_dy_Ac,
    )
    sia = dict(mask_sheet_Ac=sheet_Ac.astype(np.int32), Hi_Ac=Hi_Ac, dHs_dx_Ac=dHs_dx_Ac, dHs_dy_Ac=dHs_dy_Ac,
               dHs_dp_Ac=dHs_dp_Ac, dHs_do_Ac=dHs_do_Ac, A_flow_Ac=np.full((mesh.nAc, nZ), A, order="F"))
    return ssa, sia


def ensemble_sizes(n_members, seed=20261210, lo=2000, hi=50000):
    """Vertex counts drawn log-uniformly from [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_members)).astype(np.int64)


def ensemble_member(n_vertices, seed):
    """One member of a friction/geometry ensemble: a mesh of about ``n_vertices`` vertices,
    a dome with H0 drawn uniformly from [2000, 4000] m, and log(beta^2) a Gaussian random
    field (mean ln 1e3, std 1.0, correlation length 100 km). Returns (base, mesh, ssa)."""
    from . import api
    from .meshgen import sized_mesh
    base = sized_mesh(int(n_vertices), int(seed))
    mesh = api.build_aaac(base)
    H0 = np.random.default_rng(int(seed)).uniform(2000.0, 4000.0)
    Hi, Hb, SL = dome_geometry(base, H0=H0)
    ssa, _ = prepare_inputs(mesh, Hi, Hb, SL)
    ssa["beta_sq_AaAc"] = np.exp(log_beta_field(mesh, std=1.0, ell=100e3, seed=int(seed) + 1))
    return base, mesh, ssa


def areas_and_widths(base):
    """Per-vertex cell areas A (nV) and connection widths Cw (nV, nC_mem) for the thickness
    update, from the triangulation: A = a third of the adjacent triangle areas, Cw = the
    distance between the centroids of the two triangles on either side of a connection (to
    the edge midpoint on the domain boundary). Stand-ins for the reference's Voronoi cell
    areas and circumcentre-to-circumcentre widths, with the same units and meaning."""
    V = np.asarray(base.V, dtype=np.float64)
    T = np.asarray(base.Tri, dtype=np.int64) - 1
    p0, p1, p2 = V[T[:, 0]], V[T[:, 1]], V[T[:, 2]]
    area = 0.5 * np.abs((p1[:, 0] - p0[:, 0]) * (p2[:, 1] - p0[:, 1]) - (p2[:, 0] - p0[:, 0]) * (p1[:, 1] - p0[:, 1]))
    A = np.zeros(base.nV)
    for k in range(3):
        np.add.at(A, T[:, k], area / 3.0)
    cen = (p0 + p1 + p2) / 3.0
    nV = base.nV
    # every triangle side as a sorted vertex pair key, with its triangle
    ea = np.concatenate([T[:, 0], T[:, 1], T[:, 2]])
    eb = np.concatenate([T[:, 1], T[:, 2], T[:, 0]])
    key = np.minimum(ea, eb) * nV + np.maximum(ea, eb)
    tri = np.tile(np.arange(T.shape[0]), 3)
    order = np.argsort(key, kind="stable")
    key, tri = key[order], tri[order]
    C = np.asarray(base.C, dtype=np.int64) - 1
    nC = np.asarray(base.nC, dtype=np.int64)
    Cw = np.zeros(C.shape, order="F")
    slot = np.arange(C.shape[1])[None, :]
    valid = slot < nC[:, None]
    vv = np.repeat(np.arange(nV), C.shape[1]).reshape(C.shape)[valid]
    jj = C[valid]
    k = np.minimum(vv, jj) * nV + np.maximum(vv, jj)
    i0 = np.searchsorted(key, k, side="left")
    i1 = np.searchsorted(key, k, side="right")
    t0 = tri[i0]
    two = (i1 - i0) == 2
    t1 = np.where(two, tri[np.minimum(i0 + 1, key.size - 1)], t0)
    far = np.where(two[:, None], cen[t1], 0.5 * (V[vv] + V[jj]))
    Cw[valid] = np.linalg.norm(cen[t0] - far, axis=1)
    return A, Cw
