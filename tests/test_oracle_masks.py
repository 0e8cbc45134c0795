"""The oracle's full determine_masks (general_ice_model_data_module.f90:97-297) on CPU: the
ocean / ice / sheet / shelf masks and the Ac grounding-line mask equal those of the geometry
preparation (which the device reproduces bit for bit), and every other mask and the combined type
mask follow their definitions, recomputed here independently from the neighbour lists and the
Ac edges' two vertices (the type is the last one the routine assigns: calving front over
grounding line over margin over coast over shelf or sheet over ocean over land)."""
import numpy as np
import pytest

from conftest import oracle_aaac

import oracle as orc
from ufemism_gb300 import workloads as wl


@pytest.fixture(scope="module", params=["dome", "marine"])
def case(request):
    m = oracle_aaac("1k")
    if request.param == "dome":
        Hi, Hb, SL = wl.dome_geometry(m.base)
    else:
        Hi, Hb, SL = wl.marine_geometry(m.base, seed=20261206)
    return m, Hi, Hb, SL, orc.determine_masks(m, Hi, Hb, SL), orc.update_geometry(m, Hi, Hb, SL)


def _type(land, ocean, sheet, shelf, coast, margin, gl, cf):
    t = np.where(ocean == 1, 1, 0)
    t = np.where(sheet == 1, 3, t)
    t = np.where(shelf == 1, 4, t)
    t = np.where(coast == 1, 5, t)
    t = np.where(margin == 1, 6, t)
    t = np.where(gl == 1, 7, t)
    return np.where(cf == 1, 8, t)


def test_masks_agree_with_geometry_preparation(case):
    m, Hi, Hb, SL, M, g = case
    for k in ("mask_ocean", "mask_ice", "mask_sheet", "mask_shelf", "mask_ocean_Ac", "mask_ice_Ac", "mask_sheet_Ac",
              "mask_shelf_Ac", "mask_gl_Ac"):
        assert np.array_equal(M[k], np.asarray(g[k]).astype(np.int32)), k
    assert np.array_equal(M["mask_land"], 1 - M["mask_ocean"])
    assert np.array_equal(M["mask_land_Ac"], 1 - M["mask_ocean_Ac"])
    assert not M["mask_lake"].any() and not M["mask_lake_Ac"].any()


def test_aa_neighbour_masks_and_type(case):
    m, Hi, Hb, SL, M, g = case
    base = m.base
    nC = np.asarray(base.nC)
    C = np.asarray(base.C) - 1
    valid = np.arange(C.shape[1])[None, :] < nC[:, None]

    def any_nbr(flag):
        return np.any(valid & (flag[np.where(valid, C, 0)] == 1), axis=1).astype(np.int32)

    land, ocean, ice = M["mask_land"], M["mask_ocean"], M["mask_ice"]
    sheet, shelf = M["mask_sheet"], M["mask_shelf"]
    coast = land * any_nbr(ocean)
    margin = ice * any_nbr(1 - ice)
    gl = sheet * any_nbr(shelf)
    cf = ice * any_nbr(ocean)
    for k, v in (("coast", coast), ("margin", margin), ("gl", gl), ("cf", cf)):
        assert np.array_equal(M["mask_" + k], v), k
    assert np.array_equal(M["mask_type"], _type(land, ocean, sheet, shelf, coast, margin, gl, cf))


def test_ac_edge_masks_and_type(case):
    m, Hi, Hb, SL, M, g = case
    Aci = np.asarray(m.Aci) - 1
    vi, vj = Aci[:, 0], Aci[:, 1]

    def either(a, b):
        return ((a[vi] == 1) & (b[vj] == 1)) | ((a[vj] == 1) & (b[vi] == 1))

    land, ocean, ice = M["mask_land"], M["mask_ocean"], M["mask_ice"]
    sheet, shelf = M["mask_sheet"], M["mask_shelf"]
    coast = either(land, ocean).astype(np.int32)
    margin = either(ice, 1 - ice).astype(np.int32)
    gl = either(sheet, shelf).astype(np.int32)
    open_ocean = ((shelf == 0) & (ocean == 1)).astype(np.int32)
    cf = either(ice, open_ocean).astype(np.int32)
    for k, v in (("coast", coast), ("margin", margin), ("gl", gl), ("cf", cf)):
        assert np.array_equal(M["mask_" + k + "_Ac"], v), k
    t = _type(M["mask_land_Ac"], M["mask_ocean_Ac"], M["mask_sheet_Ac"], M["mask_shelf_Ac"], coast, margin, gl, cf)
    assert np.array_equal(M["mask_type_Ac"], t)
    if M["mask_shelf"].any():
        assert gl.any() and cf.any()
