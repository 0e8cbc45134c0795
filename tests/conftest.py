"""Shared fixtures. Tests marked ``gpu`` need an sm_103a device; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU (run with -m gpu)")


_MESHES = {}


def base_mesh(name):
    from ufemism_gb300.meshgen import dome_mesh
    if name not in _MESHES:
        _MESHES[name] = dome_mesh(name)
    return _MESHES[name]


_AAAC = {}


def oracle_aaac(name):
    import oracle as orc
    if name not in _AAAC:
        _AAAC[name] = orc.build_aaac(base_mesh(name))
    return _AAAC[name]


def oracle_inputs(m, kind="dome", seed=20261206):
    """SSA and SIA inputs on an oracle mesh, with the geometry prepared by the oracle's
    restatement of update_general_ice_model_data."""
    import oracle as orc
    from ufemism_gb300 import workloads as wl
    base = m.base
    if kind == "dome":
        Hi, Hb, SL = wl.dome_geometry(base)
    elif kind == "marine":
        Hi, Hb, SL = wl.marine_geometry(base, seed=seed)
    else:
        raise ValueError(kind)
    g = orc.update_geometry(m, Hi, Hb, SL)
    A = wl.A_FLOW
    ssa = dict(Hi=Hi, Hb=Hb, SL=SL, dHs_dx_shelf=g["dHs_dx_shelf"], dHs_dy_shelf=g["dHs_dy_shelf"],
               A_flow_mean=np.full(base.nV, A), mask_sheet=g["mask_sheet"], Hi_Ac=g["Hi_Ac"], Hb_Ac=g["Hb_Ac"],
               SL_Ac=g["SL_Ac"], dHs_dx_shelf_Ac=g["dHs_dx_shelf_Ac"], dHs_dy_shelf_Ac=g["dHs_dy_shelf_Ac"],
               A_flow_mean_Ac=np.full(m.nAc, A), mask_gl_Ac=g["mask_gl_Ac"], dHi_dx_Ac=g["dHi_dx_Ac"],
               dHi_dy_Ac=g["dHi_dy_Ac"], dSL_dx_Ac=g["dSL_dx_Ac"], dSL_dy_Ac=g["dSL_dy_Ac"],
               dHb_dx_Ac=g["dHb_dx_Ac"], dHb_dy_Ac=g["dHb_dy_Ac"])
    sia = dict(mask_sheet_Ac=g["mask_sheet_Ac"], Hi_Ac=g["Hi_Ac"], dHs_dx_Ac=g["dHs_dx_Ac"],
               dHs_dy_Ac=g["dHs_dy_Ac"], dHs_dp_Ac=g["dHs_dp_Ac"], dHs_do_Ac=g["dHs_do_Ac"],
               A_flow_Ac=np.full((m.nAc, 15), A, order="F"))
    return ssa, sia, g


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def dummy_mesh():
    """The reference's five-vertex, four-triangle dummy mesh on [-1,1]^2
    (initialise_dummy_mesh, mesh_creation_module.f90:1896-2000), in its exact arrays."""
    from ufemism_gb300.meshgen import BaseMesh, NC_MEM
    V = np.array([[-1.0, -1.0], [1.0, -1.0], [1.0, 1.0], [-1.0, 1.0], [0.0, 0.0]])
    C = np.zeros((5, NC_MEM), dtype=np.int32)
    C[0, :3] = [2, 5, 4]
    C[1, :3] = [3, 5, 1]
    C[2, :3] = [4, 5, 2]
    C[3, :3] = [1, 5, 3]
    C[4, :4] = [1, 2, 3, 4]
    iTri = np.zeros((5, NC_MEM), dtype=np.int32)
    iTri[0, :2] = [1, 4]
    iTri[1, :2] = [2, 1]
    iTri[2, :2] = [3, 2]
    iTri[3, :2] = [4, 3]
    iTri[4, :4] = [1, 2, 3, 4]
    Tri = np.array([[1, 2, 5], [2, 3, 5], [3, 4, 5], [4, 1, 5]], dtype=np.int32)
    return BaseMesh(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, V=np.asfortranarray(V),
                    nC=np.array([3, 3, 3, 3, 4], dtype=np.int32), C=np.asfortranarray(C),
                    niTri=np.array([2, 2, 2, 2, 4], dtype=np.int32), iTri=np.asfortranarray(iTri),
                    Tri=np.asfortranarray(Tri), edge_index=np.array([6, 4, 2, 8, 0], dtype=np.int32))


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
