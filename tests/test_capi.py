"""The C-ABI library loads and exports every entry point include/ufemism_gb300.h declares;
host-side validation works without a GPU (no compute call is made here)."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

from conftest import ROOT, have_gpu, oracle_aaac

from ufemism_gb300 import _native as nat
from ufemism_gb300 import api

HEADER = os.path.join(ROOT, "include", "ufemism_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ufe_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = nat.load()
    syms = declared_symbols()
    assert "ufe_ssa_solve" in syms and "ufe_sia_solve" in syms and "ufe_mesh_create" in syms
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(nat.PROTOTYPES), "ctypes prototypes out of date with the header"


def test_struct_layouts_match_header():
    # field counts of the POD structs (a cheap guard against header/binding drift)
    text = open(HEADER).read()
    for cname, py in (("ufe_params", nat.Params), ("ufe_ssa_stats", nat.SsaStats),
                      ("ufe_batch_config", nat.BatchConfig), ("ufe_batch_timing", nat.BatchTiming),
                      ("ufe_physprop_out", nat.PhyspropOut), ("ufe_triangle_mesh", nat.TriangleMesh),
                      ("ufe_sia3d_out", nat.Sia3dOut), ("ufe_geometry_out", nat.GeometryOut),
                      ("ufe_mask_out", nat.MaskOut), ("ufe_vjp_out", nat.VjpOut)):
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (cname, cname), text, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        names = re.findall(r"(\w+)(?:\[\d+\])?\s*[,;]", body)
        assert [f[0] for f in py._fields_] == names, cname


@pytest.mark.skipif(have_gpu(), reason="checks the no-device path")
def test_no_device_reported_without_gpu():
    assert nat.load().ufe_init(0) == nat.UFE_NO_DEVICE


def _desc(m, **override):
    arrs = dict(V=np.asfortranarray(m.base.V), nC=m.base.nC.astype(np.int32), iAci=m.iAci, Aci=m.Aci,
                edge_index=m.base.edge_index.astype(np.int32), edge_index_Ac=m.edge_index_Ac, nCAaAc=m.nCAaAc,
                CAaAc=m.CAaAc, Nx_AaAc=m.Nx_AaAc, Ny_AaAc=m.Ny_AaAc, Nxx_AaAc=m.Nxx_AaAc, Nxy_AaAc=m.Nxy_AaAc,
                Nyy_AaAc=m.Nyy_AaAc, colour=m.colour, colour_vi=m.colour_vi, colour_nV=m.colour_nV)
    arrs.update(override)
    keep = {k: np.asfortranarray(v) for k, v in arrs.items()}
    d = nat.MeshDesc(m.base.nV, m.nAc, m.nVAaAc, m.CAaAc.shape[1],
                     *(keep[k].ctypes.data for k in ("V", "nC", "iAci", "Aci", "edge_index", "edge_index_Ac",
                                                     "nCAaAc", "CAaAc", "Nx_AaAc", "Ny_AaAc", "Nxx_AaAc",
                                                     "Nxy_AaAc", "Nyy_AaAc", "colour", "colour_vi", "colour_nV")))
    return d, keep


def _create(d):
    h = ct.c_void_p()
    rc = nat.load().ufe_mesh_create(ct.byref(d), ct.byref(h))
    if rc == nat.UFE_OK:
        nat.load().ufe_mesh_destroy(h)
    return rc


def test_malformed_mesh_rejected_on_host():
    m = oracle_aaac("tiny")
    bad = m.CAaAc.copy()
    bad[10, 0] = m.nVAaAc + 7              # neighbour out of range
    d, keep = _desc(m, CAaAc=bad)
    assert _create(d) == nat.UFE_BAD_MESH
    col = m.colour.copy()
    vi = m.colour_vi.copy()
    # two adjacent rows in one colour: move row CAaAc(1,1) into row 1's colour list
    d, keep = _desc(m, colour_nV=np.array([m.nVAaAc, 0, 0, 0, 0], dtype=np.int32),
                    colour_vi=np.asfortranarray(np.stack([np.arange(1, m.nVAaAc + 1)] + [np.zeros(m.nVAaAc)] * 4,
                                                         axis=1).astype(np.int32)))
    assert _create(d) == nat.UFE_BAD_MESH
    d, keep = _desc(m, colour_nV=np.array([1, 0, 0, 0, 0], dtype=np.int32))
    assert _create(d) == nat.UFE_BAD_MESH
    assert "colour" in nat.last_error()


def test_ssa_entry_points_validate_arguments():
    L = nat.load()
    ps, _z = api._params_struct(api.default_params())
    assert L.ufe_ssa_run(None, ct.byref(ps), None) == nat.UFE_BAD_ARG
    assert L.ufe_ssa_solve(None, ct.byref(ps), None, None, None, None) == nat.UFE_BAD_ARG


def test_batch_entry_points_validate_arguments():
    L = nat.load()
    ps, _z = api._params_struct(api.default_params())
    h = ct.c_void_p()
    assert L.ufe_batch_create(None, 4, None, ct.byref(h)) == nat.UFE_BAD_ARG
    m = oracle_aaac("tiny")
    d, keep = _desc(m)
    cfg = nat.BatchConfig(0, 300, 1)     # not a supported CTA size
    assert L.ufe_batch_create(ct.byref(d), 1, ct.byref(cfg), ct.byref(h)) == nat.UFE_BAD_ARG
    assert "block" in nat.last_error()
    assert L.ufe_batch_run(None, ct.byref(ps), None, None) == nat.UFE_BAD_ARG
    assert L.ufe_batch_upload(None, 0, ct.byref(ps), None, None) == nat.UFE_BAD_ARG
    assert L.ufe_batch_destroy(None) == nat.UFE_BAD_ARG


def test_ssa_buffer_helpers():
    from ufemism_gb300 import api
    b = api.ssa_buffers(10, 30, 40)
    assert set(b) == set(api.SSA_INOUT_FIELDS + api.SSA_OUT_FIELDS)
    assert b["U_SSA"].shape == (10,) and b["Up_SSA_Ac"].shape == (30,) and b["N_AaAc"].shape == (40,)
    api._check_buffers(b, 10, 30, 40)
    for bad in (np.zeros(10, dtype=np.float32), np.zeros(11), np.zeros(20)[::2]):
        with pytest.raises(ValueError):
            api._check_buffers(dict(b, U_SSA=bad), 10, 30, 40)
