"""The library's host mesh substrate (ufe_aaac_build) against the oracle: Ac numbering, AaAc
connectivity, edge indices and the five-colouring bit for bit; neighbour-function
coefficients bit for bit (same expression order, no FMA contraction)."""
import numpy as np
import pytest

from conftest import base_mesh, dummy_mesh, oracle_aaac

import oracle as orc
from ufemism_gb300 import api

INT_FIELDS = ("iAci", "Aci", "edge_index_Ac", "nCAaAc", "CAaAc", "colour", "colour_vi", "colour_nV")
FP_FIELDS = ("Nx", "Ny", "Nxx", "Nxy", "Nyy", "VAc", "Nx_Ac", "Ny_Ac", "No_Ac", "Np_Ac", "VAaAc",
             "Nx_AaAc", "Ny_AaAc", "Nxx_AaAc", "Nxy_AaAc", "Nyy_AaAc")


def _bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    # NaNs (corner rows with two neighbours, as in the reference) compare by position
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.int64), b[~nb].view(np.int64))


def _compare(prod, ref):
    for k in INT_FIELDS:
        assert np.array_equal(np.asarray(getattr(prod, k)), np.asarray(getattr(ref, k))), k
    for k in FP_FIELDS:
        assert _bits_equal(getattr(prod, k), getattr(ref, k)), k


def test_dummy_mesh_bit_exact():
    b = dummy_mesh()
    _compare(api.build_aaac(b), orc.build_aaac(b))


@pytest.mark.parametrize("name", ["tiny", "1k", "4k", "16k"])
def test_dome_meshes_bit_exact(name):
    ref = oracle_aaac(name)
    assert ref.colour_status == orc.OR_OK
    _compare(api.build_aaac(base_mesh(name)), ref)


def test_ensemble_meshes_bit_exact():
    from ufemism_gb300.meshgen import sized_mesh
    for seed, n in ((11, 2000), (12, 3500)):
        b = sized_mesh(n, seed)
        ref = orc.build_aaac(b)
        assert ref.colour_status == orc.OR_OK
        _compare(api.build_aaac(b), ref)
