"""The oracle's ice_physical_properties on CPU against closed forms: the Arrhenius law on both
sides of 263.15 K, the Pounder heat capacity, the Ritz conductivity, the pressure-melting
point, Ti_Ac as the mean of the edge's two vertices, the vertical average of a profile (a
constant profile averages to itself), the shelf rule for A_flow_mean, and the two benchmark
laws (EISMINT-type constants, the MISMIP_mod time schedule)."""
import numpy as np
import pytest

from conftest import oracle_aaac

import oracle as orc
from ufemism_gb300 import workloads as wl

T0, CC, SMT, SEC = 273.16, 8.7e-4, 271.15, 31556943.36


def arrhenius(T):
    T = np.asarray(T, dtype=np.float64)
    return np.where(T < 263.15, 1.14e-5 * np.exp(-6.0e4 / (8.314 * T)), 5.47e10 * np.exp(-13.9e4 / (8.314 * T)))


@pytest.fixture(scope="module")
def case():
    m = oracle_aaac("1k")
    Hi, Hb, SL = wl.marine_geometry(m.base, seed=20261206)
    g = orc.update_geometry(m, Hi, Hb, SL)
    rng = np.random.default_rng(11)
    nV = m.base.nV
    Ti = np.asfortranarray(240.0 + 30.0 * rng.random((nV, 15)))   # both sides of 263.15 K
    return m, Hi, g, Ti


def test_arrhenius_and_parameterisations(case):
    m, Hi, g, Ti = case
    o = orc.ice_physical_properties(m, Hi, g["mask_sheet"], g["mask_sheet_Ac"], Ti)
    z = orc.ZETA_DEFAULT
    assert np.allclose(o["A_flow"], arrhenius(Ti), rtol=1e-13, atol=0)
    assert np.allclose(o["Cpi"], 2115.3 + 7.79293 * (Ti - T0), rtol=1e-14, atol=0)
    assert np.allclose(o["Ki"], 3.101e8 * np.exp(-0.0057 * Ti), rtol=1e-13, atol=0)
    assert np.allclose(o["Ti_pmp"], T0 - CC * Hi[:, None] * z[None, :], rtol=1e-15, atol=0)
    Aci = np.asarray(m.Aci) - 1
    assert np.array_equal(o["Ti_Ac"], (Ti[Aci[:, 0]] + Ti[Aci[:, 1]]) / 2.0)
    assert np.allclose(o["A_flow_Ac"], arrhenius(o["Ti_Ac"]), rtol=1e-13, atol=0)


def test_vertical_average_and_shelf_rule(case):
    m, Hi, g, Ti = case
    o = orc.ice_physical_properties(m, Hi, g["mask_sheet"], g["mask_sheet_Ac"], Ti)
    z = orc.ZETA_DEFAULT
    w = np.diff(z)
    sheet = g["mask_sheet"] == 1
    assert sheet.any() and (~sheet).any()
    avg = ((o["A_flow"][:, 1:] + o["A_flow"][:, :-1]) * 0.5 * w[None, :]).sum(axis=1)
    assert np.allclose(o["A_flow_mean"][sheet], avg[sheet], rtol=1e-13, atol=0)
    assert np.allclose(o["A_flow_mean"][~sheet], arrhenius((Ti[~sheet, 0] + SMT) / 2.0), rtol=1e-13, atol=0)
    sheet_ac = g["mask_sheet_Ac"] == 1
    avg_ac = ((o["A_flow_Ac"][:, 1:] + o["A_flow_Ac"][:, :-1]) * 0.5 * w[None, :]).sum(axis=1)
    assert np.allclose(o["A_flow_mean_Ac"][sheet_ac], avg_ac[sheet_ac], rtol=1e-13, atol=0)
    assert np.allclose(o["A_flow_mean_Ac"][~sheet_ac], arrhenius((o["Ti_Ac"][~sheet_ac, 0] + SMT) / 2.0),
                       rtol=1e-13, atol=0)
    # a constant temperature profile averages to its own flow factor
    Tc = np.asfortranarray(np.full_like(Ti, 250.0))
    oc = orc.ice_physical_properties(m, Hi, g["mask_sheet"], g["mask_sheet_Ac"], Tc)
    assert np.allclose(oc["A_flow_mean"][sheet], arrhenius(250.0), rtol=1e-14, atol=0)


def test_benchmark_laws(case):
    m, Hi, g, Ti = case
    e = orc.ice_physical_properties(m, Hi, g["mask_sheet"], g["mask_sheet_Ac"], None, flow_law=1)
    for k in ("A_flow", "A_flow_Ac", "A_flow_mean", "A_flow_mean_Ac"):
        assert np.all(e[k] == 1e-16), k
    assert np.all(e["Ki"] == 2.1 * SEC) and np.all(e["Cpi"] == 2009.0)
    z = orc.ZETA_DEFAULT
    assert np.array_equal(e["Ti_pmp"], T0 - (z[None, :] * Hi[:, None] * 8.7e-4))
    assert np.all(np.isnan(e["Ti_Ac"]))          # not written by the benchmark branch
    for t, A in ((0.0, 1e-16), (24999.0, 1e-16), (25000.0, 1e-17), (49999.0, 1e-17), (50000.0, 1e-16),
                 (80000.0, 1e-16)):
        o = orc.ice_physical_properties(m, Hi, g["mask_sheet"], g["mask_sheet_Ac"], None, flow_law=2, time=t)
        for k in ("A_flow", "A_flow_Ac", "A_flow_mean", "A_flow_mean_Ac"):
            assert np.all(o[k] == A), (t, k)
        for k in ("Ti_pmp", "Cpi", "Ki", "Ti_Ac"):
            assert np.all(np.isnan(o[k])), (t, k)
    with pytest.raises(RuntimeError):
        orc.ice_physical_properties(m, Hi, g["mask_sheet"], g["mask_sheet_Ac"], None, flow_law=0)
