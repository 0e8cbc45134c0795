"""The Halfar and Bueler benchmarks on CPU (reference_fields_module.f90:706-792, the analytic SIA
domes the reference initialises those experiments with): the oracle's geometry preparation, SIA and
thickness update stepped explicitly on the seeded 4k-vertex mesh (30-100 km spacing). Halfar, 2000
years from t = 0 with no mass balance: the volume is conserved to rounding. Bueler with lam = 5,
1000 years from t0 with its accumulation M = lam H / t: the volume grows by exactly the SMB added.
Both follow their similarity solutions (dome within 0.5 %, 2 % relative L2 inside 0.6 R0, 5 % over
the whole ice sheet)."""
import numpy as np

from conftest import oracle_aaac

import oracle as orc
from ufemism_gb300 import workloads as wl

SEC_PER_YEAR = 31556943.36


def halfar(H0, R0, x, y, t_years):
    """Halfar_solution (reference_fields_module.f90:706-744): A = 1e-16 Pa^-3 yr^-1, n = 3."""
    A, rho, g = 1e-16, 910.0, 9.81
    gamma = (2.0 / 5.0) * (A / SEC_PER_YEAR) * (rho * g) ** 3.0
    t0 = 1.0 / (18.0 * gamma) * (7.0 / 4.0) ** 3.0 * R0 ** 4.0 / H0 ** 7.0
    tp = t_years * SEC_PER_YEAR + t0
    r = np.sqrt(x * x + y * y)
    f1 = (t0 / tp) ** (1.0 / 9.0)
    f2 = (t0 / tp) ** (1.0 / 18.0)
    return H0 * f1 * np.maximum(0.0, 1.0 - (f2 * r / R0) ** (4.0 / 3.0)) ** (3.0 / 7.0)


def test_halfar_dome_sia_and_thickness_update():
    m = oracle_aaac("4k")
    base = m.base
    x, y = base.V[:, 0], base.V[:, 1]
    H0, R0, dt, T = 3000.0, 500e3, 2.0, 2000.0
    Hi = halfar(H0, R0, x, y, 0.0)
    Hb = np.zeros(base.nV)
    SL = np.zeros(base.nV)
    Aw, Cw = wl.areas_and_widths(base)
    p = orc.default_params()
    A = np.full((m.nAc, 15), 1e-16, order="F")
    zac, zv = np.zeros(m.nAc), np.zeros(base.nV)
    V0 = np.sum(Aw * Hi)
    for _ in range(int(round(T / dt))):
        g = orc.update_geometry(m, Hi, Hb, SL)
        sia = dict(mask_sheet_Ac=g["mask_sheet_Ac"], Hi_Ac=g["Hi_Ac"], dHs_dx_Ac=g["dHs_dx_Ac"],
                   dHs_dy_Ac=g["dHs_dy_Ac"], dHs_dp_Ac=g["dHs_dp_Ac"], dHs_do_Ac=g["dHs_do_Ac"], A_flow_Ac=A)
        up = orc.solve_sia(m, sia, p)["Up_SIA_Ac"]
        Hi = orc.thickness_change(m, Aw, Cw, up, zac, zv, zv, dt, Hi)[0]
    He = halfar(H0, R0, x, y, T)
    assert abs(np.sum(Aw * Hi) / V0 - 1.0) < 1e-12
    c = np.argmin(np.hypot(x, y))
    assert abs(Hi[c] / He[c] - 1.0) < 5e-3, (Hi[c], He[c])
    inner = np.hypot(x, y) < 0.6 * R0
    assert np.linalg.norm((Hi - He)[inner]) / np.linalg.norm(He[inner]) < 0.02
    assert np.linalg.norm(Hi - He) / np.linalg.norm(He) < 0.05
    assert np.all(Hi >= 0.0)


def bueler(H0, R0, lam, x, y, t_years):
    """Bueler_solution (reference_fields_module.f90:745-792), with the surface mass balance
    M = lam H / t that drives it; returns (H, t0 in years)."""
    A, rho, g, n = 1e-16, 910.0, 9.81, 3.0
    alpha = (2.0 - (n + 1.0) * lam) / (5.0 * n + 3.0)
    beta = (1.0 + (2.0 * n + 1.0) * lam) / (5.0 * n + 3.0)
    gamma = 2.0 / 5.0 * (A / SEC_PER_YEAR) * (rho * g) ** n
    t0 = (beta / gamma) * ((2.0 * n + 1.0) / (n + 1.0)) ** n * R0 ** (n + 1.0) / H0 ** (2.0 * n + 1.0)
    tp = t_years * SEC_PER_YEAR
    f3 = np.sqrt(x * x + y * y) / R0
    f4 = np.maximum(0.0, 1.0 - ((tp / t0) ** (-beta) * f3) ** ((n + 1.0) / n))
    return H0 * (tp / t0) ** (-alpha) * f4 ** (n / (2.0 * n + 1.0)), t0 / SEC_PER_YEAR


def test_bueler_dome_with_accumulation():
    """Bueler's solution with lam = 5 (an accumulating, advancing ice sheet) from t0 for 1000
    years: the SMB term of the thickness update adds exactly its volume, and the thickness
    follows the solution (dome within 0.5 %, 2 % relative L2 inside 0.6 R0)."""
    m = oracle_aaac("4k")
    base = m.base
    x, y = base.V[:, 0], base.V[:, 1]
    H0, R0, lam, dt, T = 3000.0, 500e3, 5.0, 1.0, 1000.0
    _, t0 = bueler(H0, R0, lam, x, y, 1.0)
    Hi = bueler(H0, R0, lam, x, y, t0)[0]
    Hb = np.zeros(base.nV)
    SL = np.zeros(base.nV)
    Aw, Cw = wl.areas_and_widths(base)
    p = orc.default_params()
    A = np.full((m.nAc, 15), 1e-16, order="F")
    zac, zv = np.zeros(m.nAc), np.zeros(base.nV)
    V0, added, t = np.sum(Aw * Hi), 0.0, t0
    for _ in range(int(round(T / dt))):
        g = orc.update_geometry(m, Hi, Hb, SL)
        sia = dict(mask_sheet_Ac=g["mask_sheet_Ac"], Hi_Ac=g["Hi_Ac"], dHs_dx_Ac=g["dHs_dx_Ac"],
                   dHs_dy_Ac=g["dHs_dy_Ac"], dHs_dp_Ac=g["dHs_dp_Ac"], dHs_do_Ac=g["dHs_do_Ac"], A_flow_Ac=A)
        up = orc.solve_sia(m, sia, p)["Up_SIA_Ac"]
        tm = t + 0.5 * dt
        smb = lam / tm * bueler(H0, R0, lam, x, y, tm)[0]
        added += np.sum(Aw * smb) * dt
        Hi = orc.thickness_change(m, Aw, Cw, up, zac, smb, zv, dt, Hi)[0]
        t += dt
    He = bueler(H0, R0, lam, x, y, t)[0]
    assert abs(np.sum(Aw * Hi) / (V0 + added) - 1.0) < 1e-12
    c = np.argmin(np.hypot(x, y))
    assert abs(Hi[c] / He[c] - 1.0) < 5e-3, (Hi[c], He[c])
    inner = np.hypot(x, y) < 0.6 * R0
    assert np.linalg.norm((Hi - He)[inner]) / np.linalg.norm(He[inner]) < 0.02
    assert np.linalg.norm(Hi - He) / np.linalg.norm(He) < 0.05
