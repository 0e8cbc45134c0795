"""ufe_sia_solve_noalloc through the C-ABI (run with -m gpu).

The entry point takes device arrays and keeps its intermediates in the library's fixed
scratch array; it is compared with ufe_sia_solve (host arrays, per-handle buffers) on two
calls in a row with different inputs, so a second call cannot pass on what the first left
in the scratch. The test allocates its device arrays with torch; the entry point allocates
nothing. Tolerance: 1e-12 relative L2 (the same kernels run on the same inputs).
"""
import ctypes as ct

import numpy as np
import pytest

from conftest import base_mesh, rel_l2

from ufemism_gb300 import _native as nat
from ufemism_gb300 import api
from ufemism_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-12
AC_FIELDS = ("D_SIA_Ac", "Ux_SIA_Ac", "Uy_SIA_Ac", "Up_SIA_Ac", "Uo_SIA_Ac")
AA_FIELDS = ("U_SIA", "V_SIA", "D_SIA")
IN_FIELDS = ("mask_sheet_Ac", "Hi_Ac", "dHs_dx_Ac", "dHs_dy_Ac", "dHs_dp_Ac", "dHs_do_Ac", "A_flow_Ac")


@pytest.fixture(scope="module")
def setup():
    import torch
    api.init(0)
    base = base_mesh("4k")
    mesh = api.build_aaac(base)
    dm = api.DeviceMesh(mesh)
    yield torch, base, mesh, dm
    dm.close()


def sia_inputs(base, mesh, H0, A):
    Hi, Hb, SL = wl.dome_geometry(base, H0=H0)
    ssa, sia = wl.prepare_inputs(mesh, Hi, Hb, SL, A=A)
    return sia


def to_device(torch, sia):
    """Device copies of the SIA inputs in the reference's layout ((nAc, nZ) column-major)."""
    d = {"mask_sheet_Ac": torch.from_numpy(np.ascontiguousarray(sia["mask_sheet_Ac"], dtype=np.int32)).cuda()}
    for k in IN_FIELDS[1:6]:
        d[k] = torch.from_numpy(np.ascontiguousarray(sia[k], dtype=np.float64)).cuda()
    A = np.asfortranarray(sia["A_flow_Ac"], dtype=np.float64)
    d["A_flow_Ac"] = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()   # (nZ, nAc) row-major == (nAc, nZ) F
    return d


def device_outputs(torch, nAc, nV, nZ, ac=True, full=True):
    out = {"D_SIA_3D_Ac": torch.full((nZ, nAc), np.nan, dtype=torch.float64, device="cuda") if full else None}
    for k in AC_FIELDS:
        out[k] = torch.full((nAc,), np.nan, dtype=torch.float64, device="cuda") if ac else None
    for k in AA_FIELDS:
        out[k] = torch.full((nV,), np.nan, dtype=torch.float64, device="cuda")
    return out


def ptr(t):
    return None if t is None else t.data_ptr()


def call_noalloc(dm, params, din, dout):
    L = nat.load()
    si = nat.SiaIn(*(din[k].data_ptr() for k in IN_FIELDS))
    so = nat.SiaOut(*(ptr(dout[k]) for k in ("D_SIA_3D_Ac",) + AC_FIELDS + AA_FIELDS))
    ps, _z = api._params_struct(params)
    return L.ufe_sia_solve_noalloc(dm._h, ct.byref(ps), ct.byref(si), ct.byref(so))


def host(t):
    return t.cpu().numpy()


def test_noalloc_matches_sia_solve_twice(setup):
    torch, base, mesh, dm = setup
    p = api.default_params()
    nZ = len(p["zeta"])
    for H0, A in ((3600.0, 1e-16), (2400.0, 3e-16)):
        sia = sia_inputs(base, mesh, H0, A)
        ref = dm.solve_sia(sia, p)
        din = to_device(torch, sia)
        dout = device_outputs(torch, mesh.nAc, base.nV, nZ)
        torch.cuda.synchronize()
        rc = call_noalloc(dm, p, din, dout)
        assert rc == nat.UFE_OK, nat.last_error()
        got3 = host(dout["D_SIA_3D_Ac"]).T
        assert rel_l2(got3, ref["D_SIA_3D_Ac"]) <= TOL
        for k in AC_FIELDS + AA_FIELDS:
            g = host(dout[k])
            assert np.all(np.isfinite(g)), k
            assert rel_l2(g, ref[k]) <= TOL, k


def test_noalloc_scratch_for_ac_intermediates_twice(setup):
    """Only the Aa velocities requested: the Ac fields live in the scratch. Two calls in a
    row with different inputs, each against ufe_sia_solve."""
    torch, base, mesh, dm = setup
    p = api.default_params()
    nZ = len(p["zeta"])
    for H0, A in ((3000.0, 2e-16), (3900.0, 1e-16)):
        sia = sia_inputs(base, mesh, H0, A)
        ref = dm.solve_sia(sia, p)
        din = to_device(torch, sia)
        dout = device_outputs(torch, mesh.nAc, base.nV, nZ, ac=False, full=False)
        torch.cuda.synchronize()
        rc = call_noalloc(dm, p, din, dout)
        assert rc == nat.UFE_OK, nat.last_error()
        for k in AA_FIELDS:
            assert rel_l2(host(dout[k]), ref[k]) <= TOL, k


def test_noalloc_rejects_host_arrays(setup):
    torch, base, mesh, dm = setup
    p = api.default_params()
    nZ = len(p["zeta"])
    sia = sia_inputs(base, mesh, 3600.0, 1e-16)
    din = to_device(torch, sia)
    hostHi = np.ascontiguousarray(sia["Hi_Ac"], dtype=np.float64)

    class HostArr:   # a host pointer where a device array belongs
        def data_ptr(self):
            return hostHi.ctypes.data
    din["Hi_Ac"] = HostArr()
    dout = device_outputs(torch, mesh.nAc, base.nV, nZ)
    torch.cuda.synchronize()
    rc = call_noalloc(dm, p, din, dout)
    assert rc == nat.UFE_BAD_ARG
    assert "not device memory" in nat.last_error()


def test_noalloc_rejects_mesh_beyond_scratch(setup):
    torch = setup[0]
    big = api.build_aaac(base_mesh("100k"))
    assert big.nAc > nat.UFE_SIA_NOALLOC_MAX_AC
    dm = api.DeviceMesh(big)
    try:
        p = api.default_params()
        nZ = len(p["zeta"])
        sia = {"mask_sheet_Ac": np.zeros(big.nAc, np.int32), "A_flow_Ac": np.zeros((big.nAc, nZ), order="F")}
        for k in IN_FIELDS[1:6]:
            sia[k] = np.zeros(big.nAc)
        din = to_device(torch, sia)
        dout = device_outputs(torch, big.nAc, big.base.nV, nZ)
        torch.cuda.synchronize()
        rc = call_noalloc(dm, p, din, dout)
        assert rc == nat.UFE_BAD_ARG
        assert "scratch holds at most %d" % nat.UFE_SIA_NOALLOC_MAX_AC in nat.last_error()
    finally:
        dm.close()


def test_noalloc_drops_the_handles_sia_velocities(setup):
    """After ufe_sia_solve the handle offers its Up_SIA_Ac to a thickness update given none;
    after a no-allocation call (whose results stay in the caller's arrays) it must not, so a
    thickness update without Up_SIA_Ac is refused rather than advecting with the older field."""
    torch, base, mesh, dm = setup
    p = api.default_params()
    nZ = len(p["zeta"])
    sia = sia_inputs(base, mesh, 3600.0, 1e-16)
    dm.geometry_attach(mesh)
    ref = dm.solve_sia(sia, p)
    Hi, _, _ = wl.dome_geometry(base)
    Aw, Cw = wl.areas_and_widths(base)
    smb, bmb = np.full(base.nV, 0.3), np.zeros(base.nV)
    up_ssa = np.zeros(mesh.nAc)
    h1 = dm.thickness_update(Hi, Aw, Cw, smb, bmb, 10.0, Up_SSA_Ac=up_ssa)[0]
    h2 = dm.thickness_update(Hi, Aw, Cw, smb, bmb, 10.0, Up_SIA_Ac=ref["Up_SIA_Ac"], Up_SSA_Ac=up_ssa)[0]
    assert np.array_equal(h1, h2)
    din = to_device(torch, sia_inputs(base, mesh, 2400.0, 3e-16))
    dout = device_outputs(torch, mesh.nAc, base.nV, nZ)
    torch.cuda.synchronize()
    assert call_noalloc(dm, p, din, dout) == nat.UFE_OK, nat.last_error()
    with pytest.raises(nat.UfeError) as e:
        dm.thickness_update(Hi, Aw, Cw, smb, bmb, 10.0, Up_SSA_Ac=up_ssa)
    assert e.value.status == nat.UFE_BAD_ARG
    got = dm.thickness_update(Hi, Aw, Cw, smb, bmb, 10.0, Up_SIA_Ac=host(dout["Up_SIA_Ac"]), Up_SSA_Ac=up_ssa)[0]
    assert np.all(np.isfinite(got))
