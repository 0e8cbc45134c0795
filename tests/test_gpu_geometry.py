"""Geometry preparation on the device (run with -m gpu): every derived field bit-identical to
the oracle's restatement of update_general_ice_model_data, and a solve fed by the device
geometry identical to one fed by host-prepared fields."""
import numpy as np
import pytest

from conftest import oracle_aaac, oracle_inputs, rel_l2

import oracle as orc
from ufemism_gb300 import _native as nat
from ufemism_gb300 import api
from ufemism_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def device():
    api.init(0)


@pytest.mark.parametrize("kind", ["dome", "marine"])
def test_device_geometry_bit_identical_to_oracle(kind):
    m = oracle_aaac("4k")
    base = m.base
    Hi, Hb, SL = wl.dome_geometry(base) if kind == "dome" else wl.marine_geometry(base, seed=20261206)
    ref = orc.update_geometry(m, Hi, Hb, SL)
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    got = dm.geometry_update(Hi, Hb, SL)
    for k in nat.GEOM_OUT_FIELDS:
        assert np.array_equal(got[k], np.asarray(ref[k]).astype(got[k].dtype)), k
    if kind == "marine":
        assert got["mask_gl_Ac"].sum() > 0 and got["mask_shelf"].sum() > 0
    dm.close()


@pytest.mark.parametrize("kind,size", [("dome", "4k"), ("marine", "4k"), ("marine", "100k")])
def test_device_masks_bit_identical_to_oracle(kind, size):
    """determine_masks in full on the device (land, ocean, lake, ice, sheet, shelf, coast,
    margin, grounding line, calving front and the type mask, on Aa and Ac) against the
    oracle's literal restatement, after a geometry update and again after the solve's own
    geometry upload (the masks are born and stay on the device)."""
    m = oracle_aaac(size)
    base = m.base
    Hi, Hb, SL = wl.dome_geometry(base) if kind == "dome" else wl.marine_geometry(base, seed=20261206)
    ref = orc.determine_masks(m, Hi, Hb, SL)
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    dm.geometry_update(Hi, Hb, SL)
    got = dm.geometry_masks()
    for name in orc.MASK_NAMES:
        k = "mask" if name == "type" else "mask_" + name
        assert np.array_equal(got[k], ref["mask_" + name]), k
        assert np.array_equal(got[k + "_Ac"], ref["mask_" + name + "_Ac"]), k + "_Ac"
    if kind == "marine":
        for k in ("mask_coast", "mask_gl", "mask_cf", "mask_margin", "mask_gl_Ac", "mask_cf_Ac"):
            assert got[k].sum() > 0, k
        # the type is the last assignment in the routine's order: calving front wins over
        # grounding line, margin and shelf where they coincide
        assert {1, 3, 8} <= set(np.unique(got["mask"])) and len(np.unique(got["mask_Ac"])) >= 4
    # the SSA's own geometry upload recomputes them from other thickness fields
    Hi2 = np.where(Hi > 0, Hi * 0.8, 0.0)
    p = api.default_params(precision=nat.UFE_MIXED)
    dm.ssa_upload_geometry(Hi2, Hb, SL, np.full(base.nV, wl.A_FLOW), np.full(m.nAc, wl.A_FLOW), p)
    ref2 = orc.determine_masks(m, Hi2, Hb, SL)
    got2 = dm.geometry_masks()
    assert np.array_equal(got2["mask"], ref2["mask_type"]) and np.array_equal(got2["mask_Ac"], ref2["mask_type_Ac"])
    assert np.array_equal(got2["mask_cf"], ref2["mask_cf"])
    dm.close()


def test_solve_from_device_geometry_matches_host_fields():
    m = oracle_aaac("4k")
    ssa, sia, g = oracle_inputs(m, "marine")
    beta = np.exp(wl.log_beta_field(m, std=1.0, ell=100e3, seed=3))
    p = api.default_params(precision=nat.UFE_FP64)
    dm = api.DeviceMesh(m)
    f = dict(ssa, beta_sq_AaAc=beta)
    rc1, o1, s1 = dm.solve_ssa(f, p)
    dm.geometry_attach(m)
    dm.ssa_upload_geometry(ssa["Hi"], ssa["Hb"], ssa["SL"], ssa["A_flow_mean"], ssa["A_flow_mean_Ac"], p, beta=beta)
    rc2, s2 = dm.ssa_run(p)
    o2 = dm.ssa_download()
    assert rc2 == rc1 and s2["sweeps"] == s1["sweeps"]
    for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "N_AaAc"):
        assert np.array_equal(o2[k], o1[k]), k
    dm.close()


def test_geometry_attach_rejects_bad_indices():
    m = oracle_aaac("tiny")
    dm = api.DeviceMesh(m)

    class Bad:
        pass
    bad = Bad()
    for k in ("base", "Nx", "Ny", "Aci", "Nx_Ac", "Ny_Ac", "No_Ac", "Np_Ac", "CAaAc"):
        setattr(bad, k, getattr(m, k))
    b2 = Bad()
    b2.nC, b2.C = m.base.nC, m.base.C.copy()
    b2.C[3, 0] = m.base.nV + 10
    bad.base = b2
    with pytest.raises(nat.UfeError) as e:
        dm.geometry_attach(bad)
    assert e.value.status == nat.UFE_BAD_MESH
    dm.close()


def _thickness_case(name="4k"):
    m = oracle_aaac(name)
    ssa, sia, g = oracle_inputs(m, "marine")
    A, Cw = wl.areas_and_widths(m.base)
    rng = np.random.default_rng(11)
    up_sia = rng.normal(size=m.nAc) * 50.0
    up_ssa = rng.normal(size=m.nAc) * 400.0
    smb = rng.normal(size=m.base.nV) * 0.5
    bmb = -np.abs(rng.normal(size=m.base.nV)) * 20.0 * (ssa["Hi"] > 0)
    noice = (rng.uniform(size=m.base.nV) < 0.01).astype(np.int32)
    return m, ssa, A, Cw, up_sia, up_ssa, smb, bmb, noice


@pytest.mark.parametrize("dt", [10.0, 0.0, 250.0])
def test_thickness_update_bit_identical_to_oracle(dt):
    """dt = 250 yr forces outflux rescales on many vertices."""
    m, ssa, A, Cw, up_sia, up_ssa, smb, bmb, noice = _thickness_case()
    ref = orc.thickness_change(m, A, Cw, up_sia, up_ssa, smb, bmb, dt, ssa["Hi"], mask_noice=noice)
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    got = dm.thickness_update(ssa["Hi"], A, Cw, smb, bmb, dt, Up_SIA_Ac=up_sia, Up_SSA_Ac=up_ssa, mask_noice=noice)
    for k, (a, b) in enumerate(zip(got, ref)):
        assert np.array_equal(a, b), ("Hi", "Hi_prev", "dHi_dt", "dVi_in")[k]
    if dt == 250.0:
        # rescaled outfluxes leave at most rounding-level negative thickness (as the reference)
        assert np.any(got[0] == 0.0) and np.all(got[0] >= -1e-9 * ssa["Hi"].max())
    dm.close()


def test_thickness_update_from_device_velocities():
    """Velocities left on the device by the SSA and SIA solves of the same handle."""
    m, ssa, A, Cw, up_sia, up_ssa, smb, bmb, noice = _thickness_case("1k")
    sia = oracle_inputs(m, "marine")[1]
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    rc, o, st = dm.solve_ssa(ssa, api.default_params(), check=False)
    so = dm.solve_sia(sia, api.default_params())
    got = dm.thickness_update(ssa["Hi"], A, Cw, smb, bmb, 5.0)
    ref = orc.thickness_change(m, A, Cw, so["Up_SIA_Ac"], o["Up_SSA_Ac"], smb, bmb, 5.0, ssa["Hi"])
    assert np.array_equal(got[0], ref[0])
    dm.close()


def test_device_time_step_geometry_sia_ssa_thickness():
    """A whole velocity-and-thickness step on the device from Hi, Hb, SL: geometry, SIA and
    SSA solves on it, thickness update from the velocities the solves left on the device —
    identical to the same step fed with the oracle's host-prepared fields."""
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m, "marine")
    A, Cw = wl.areas_and_widths(m.base)
    rng = np.random.default_rng(2)
    smb = rng.normal(size=m.base.nV) * 0.5
    bmb = -np.abs(rng.normal(size=m.base.nV)) * 5.0 * (ssa["Hi"] > 0)
    p = api.default_params()
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    dm.ssa_upload_geometry(ssa["Hi"], ssa["Hb"], ssa["SL"], ssa["A_flow_mean"], ssa["A_flow_mean_Ac"], p)
    rc, st = dm.ssa_run(p, check=False)
    o_dev = dm.ssa_download()
    s_dev = dm.solve_sia_geometry(sia["A_flow_Ac"], p)
    H_dev = dm.thickness_update(ssa["Hi"], A, Cw, smb, bmb, 10.0)[0]
    dm2 = api.DeviceMesh(m)
    rc2, o_host, st2 = dm2.solve_ssa(ssa, p, check=False)
    s_host = dm2.solve_sia(sia, p)
    for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "Up_SSA_Ac"):
        assert np.array_equal(o_dev[k], o_host[k]), k
    for k in ("D_SIA_3D_Ac", "Up_SIA_Ac", "U_SIA", "V_SIA"):
        assert np.array_equal(s_dev[k], s_host[k]), k
    ref = orc.thickness_change(m, A, Cw, s_host["Up_SIA_Ac"], o_host["Up_SSA_Ac"], smb, bmb, 10.0, ssa["Hi"])
    assert np.array_equal(H_dev, ref[0])
    dm.close()
    dm2.close()


def test_frictional_heating_matches_oracle():
    """bottom_frictional_heating from the device solve's own U, V and tau_c against the
    oracle's restatement applied to the downloaded fields (CUDA's pow vs the C library's:
    1e-14 relative)."""
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m, "marine")
    p = api.default_params(sliding_law=nat.UFE_SLIDING_COULOMB_REGULARISED)
    dm = api.DeviceMesh(m)
    rc, o, st = dm.solve_ssa(ssa, p, check=False)
    got = dm.frictional_heating(ssa["mask_sheet"])
    nV = m.base.nV
    ref = orc.frictional_heating(ssa["mask_sheet"], o["tau_c_AaAc"][:nV], o["U_SSA"], o["V_SSA"])
    assert np.count_nonzero(ref) > 0
    assert np.allclose(got, ref, rtol=1e-14, atol=0.0)
    assert np.all(got[ssa["mask_sheet"] == 0] == 0.0)
    dm.close()


@pytest.mark.parametrize("kind", ["dome", "marine"])
def test_sia3d_matches_oracle(kind):
    """solve_SIA_3D on the device geometry and the device SSA solution against the oracle's
    restatement fed with the same fields (CUDA's pow vs the C library's: 1e-12 relative)."""
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m, kind)
    nV = m.base.nV
    rng = np.random.default_rng(4)
    A3 = np.asfortranarray(np.full((nV, 15), 1e-16) * (1.0 + 0.5 * rng.uniform(size=(nV, 1))))
    dHb_dt = rng.normal(size=nV) * 1e-3
    p = api.default_params()
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    dm.ssa_upload_geometry(ssa["Hi"], ssa["Hb"], ssa["SL"], ssa["A_flow_mean"], ssa["A_flow_mean_Ac"], p)
    dm.ssa_run(p, check=False)
    o = dm.ssa_download()
    U3, V3, W3 = dm.solve_sia_3d(A3, dHb_dt, p)
    rU, rV, rW = orc.solve_sia_3d(m, g, A3, dHb_dt, o["U_SSA"], o["V_SSA"])
    for a, b, name in ((U3, rU, "U"), (V3, rV, "V"), (W3, rW, "W")):
        assert rel_l2(a, b) <= 1e-12, name
    assert np.all(W3[m.base.edge_index == 0][g["mask_sheet"][m.base.edge_index == 0] == 0] == 0.0)
    dm.close()


@pytest.mark.parametrize("law", [nat.UFE_FLOW_ARRHENIUS, nat.UFE_FLOW_EISMINT, nat.UFE_FLOW_MISMIP_MOD])
def test_physical_properties_match_oracle(law):
    """ice_physical_properties on the device against the oracle: the fields without a
    transcendental function bit-identical, the rest within CUDA's exp against the C library's."""
    m = oracle_aaac("1k")
    Hi, Hb, SL = wl.marine_geometry(m.base, seed=20261206)
    g = orc.update_geometry(m, Hi, Hb, SL)
    rng = np.random.default_rng(12)
    Ti = np.asfortranarray(240.0 + 30.0 * rng.random((m.base.nV, 15)))
    T = Ti if law == nat.UFE_FLOW_ARRHENIUS else None
    p = api.default_params()
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    dm.geometry_update(Hi, Hb, SL)
    got = dm.ice_physical_properties(p, T, flow_law=law, time=30000.0)
    ref = orc.ice_physical_properties(m, Hi, g["mask_sheet"], g["mask_sheet_Ac"], T, flow_law=law, time=30000.0)
    assert set(got) == {k for k, v in ref.items() if not np.all(np.isnan(v))}
    for k, v in got.items():
        if k in ("Ti_Ac", "Ti_pmp", "Cpi") or law != nat.UFE_FLOW_ARRHENIUS:
            assert np.array_equal(v, ref[k]), k
        else:
            assert np.allclose(v, ref[k], rtol=1e-14, atol=0.0), k
    dm.close()


def test_physical_properties_feed_the_solves():
    """SSA, SIA and 3-D SIA fed by the flow factors left on the device equal the same solves
    fed by those values from the host; before any physical properties the NULL forms fail."""
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m, "dome")
    Hi, Hb, SL = ssa["Hi"], ssa["Hb"], ssa["SL"]
    nV = m.base.nV
    rng = np.random.default_rng(13)
    Ti = np.asfortranarray(250.0 + 15.0 * rng.random((nV, 15)))
    dHb_dt = rng.normal(size=nV) * 1e-3
    p = api.default_params(precision=nat.UFE_FP64)
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    dm.geometry_update(Hi, Hb, SL)
    with pytest.raises(nat.UfeError):
        dm.ssa_upload_geometry(Hi, Hb, SL, None, None, p)
    with pytest.raises(nat.UfeError):
        dm.solve_sia_3d(None, dHb_dt, p)
    props = dm.ice_physical_properties(p, Ti)
    runs = []
    for A in (None, props):
        dm.ssa_upload_geometry(Hi, Hb, SL, None if A is None else A["A_flow_mean"],
                               None if A is None else A["A_flow_mean_Ac"], p)
        rc, st = dm.ssa_run(p, check=False)
        o = dm.ssa_download()
        s = dm.solve_sia_geometry(None if A is None else A["A_flow_Ac"], p)
        u = dm.solve_sia_3d(None if A is None else A["A_flow"], dHb_dt, p)
        runs.append((rc, st["sweeps"], o, s, u))
    (rc1, sw1, o1, s1, u1), (rc2, sw2, o2, s2, u2) = runs
    assert rc1 == rc2 and sw1 == sw2
    for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac"):
        assert np.array_equal(o1[k], o2[k]), k
    for k in ("Ux_SIA_Ac", "Uy_SIA_Ac", "D_SIA_3D_Ac", "U_SIA"):
        assert np.array_equal(s1[k], s2[k]), k
    for a, b in zip(u1, u2):
        assert np.array_equal(a, b)
    assert np.count_nonzero(o1["U_SSA"]) > 0
    dm.close()


def _triangles(m, dm):
    NxT, NyT = orc.triangle_functions(m.base)
    R = orc.vertex_resolution(m.base)
    dm.triangles_attach(m.base, R, NxT, NyT)
    return R, NxT, NyT


def test_upwind_derivatives_match_oracle():
    """get_upwind_derivative_vertex_3D on the device: bit-identical to the oracle (same
    triangle decisions, separately rounded arithmetic), including the windless layer and the
    count of edge pairs without an upwind triangle."""
    m = oracle_aaac("4k")
    nV, nZ = m.base.nV, 15
    rng = np.random.default_rng(21)
    U = rng.normal(size=(nV, nZ)) * 200.0
    V = rng.normal(size=(nV, nZ)) * 200.0
    U[:, 3] = 0.0
    V[:, 3] = 0.0
    U, V = np.asfortranarray(U), np.asfortranarray(V)
    d = np.asfortranarray(250.0 + 20.0 * rng.random((nV, nZ)))
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    R, NxT, NyT = _triangles(m, dm)
    p = api.default_params()
    gx, gy, gmiss = dm.upwind_derivatives_3d(p, U, V, d)
    rx, ry, rmiss = orc.upwind_derivatives_3d(m, R, NxT, NyT, U, V, d)
    assert np.array_equal(gx, rx) and np.array_equal(gy, ry)
    assert gmiss == rmiss and 0 < rmiss < nV * nZ // 20
    dm.close()


def test_upwind_derivatives_of_the_device_step():
    """Ti -> physical properties -> SSA -> 3-D SIA -> upwind derivatives of Ti with every field
    left on the device, equal to the same call given those fields from the host."""
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m, "dome")
    nV = m.base.nV
    rng = np.random.default_rng(22)
    Ti = np.asfortranarray(250.0 + 15.0 * rng.random((nV, 15)))
    p = api.default_params(precision=nat.UFE_FP64)
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    _triangles(m, dm)
    dm.geometry_update(ssa["Hi"], ssa["Hb"], ssa["SL"])
    with pytest.raises(nat.UfeError):
        dm.upwind_derivatives_3d(p)          # no 3-D velocities yet
    dm.ice_physical_properties(p, Ti)
    dm.ssa_upload_geometry(ssa["Hi"], ssa["Hb"], ssa["SL"], None, None, p)
    dm.ssa_run(p, check=False)
    U3, V3, _ = dm.solve_sia_3d(None, np.zeros(nV), p)
    gx, gy, gm = dm.upwind_derivatives_3d(p)
    hx, hy, hm = dm.upwind_derivatives_3d(p, U3, V3, Ti)
    assert np.array_equal(gx, hx) and np.array_equal(gy, hy) and gm == hm
    assert np.count_nonzero(gx) > 0
    dm.close()


def test_halfar_time_loop_on_the_device():
    """The Halfar benchmark stepped on the device — geometry preparation, the SIA on the device
    geometry, the thickness update taking the SIA velocities from the device — against the same
    loop of the oracle (CUDA's pow in the SIA against the C library's: 1e-10 after 200 steps)."""
    from test_oracle_halfar import halfar
    m = oracle_aaac("4k")
    base = m.base
    x, y = base.V[:, 0], base.V[:, 1]
    dt, steps = 2.0, 200
    H0 = halfar(3000.0, 500e3, x, y, 0.0)
    Hb, SL = np.zeros(base.nV), np.zeros(base.nV)
    Aw, Cw = wl.areas_and_widths(base)
    A = np.full((m.nAc, 15), 1e-16, order="F")
    zac, zv = np.zeros(m.nAc), np.zeros(base.nV)
    p = api.default_params()
    dm = api.DeviceMesh(m)
    dm.geometry_attach(m)
    Hd = H0.copy()
    for _ in range(steps):
        dm.geometry_update(Hd, Hb, SL)
        dm.solve_sia_geometry(A, p)
        Hd = dm.thickness_update(Hd, Aw, Cw, zv, zv, dt, Up_SSA_Ac=zac)[0]
    dm.close()
    Ho = H0.copy()
    po = orc.default_params()
    for _ in range(steps):
        g = orc.update_geometry(m, Ho, Hb, SL)
        sia = dict(mask_sheet_Ac=g["mask_sheet_Ac"], Hi_Ac=g["Hi_Ac"], dHs_dx_Ac=g["dHs_dx_Ac"],
                   dHs_dy_Ac=g["dHs_dy_Ac"], dHs_dp_Ac=g["dHs_dp_Ac"], dHs_do_Ac=g["dHs_do_Ac"], A_flow_Ac=A)
        up = orc.solve_sia(m, sia, po)["Up_SIA_Ac"]
        Ho = orc.thickness_change(m, Aw, Cw, up, zac, zv, zv, dt, Ho)[0]
    assert rel_l2(Hd, Ho) <= 1e-10
    assert abs(np.sum(Aw * Hd) / np.sum(Aw * H0) - 1.0) < 1e-12
