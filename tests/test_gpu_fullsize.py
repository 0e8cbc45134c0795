"""The benchmark workload itself against the oracle (run with -m gpu).

The 200k-vertex dome (about 810k AaAc rows, 4.85M neighbour entries) is the size the headline
solves/s is quoted on. The oracle's full cold-start FP64 solve of it runs once per module on
every host core (about a minute and a half on 16 cores), and each GPU path is checked against
that one result:

* FP64 in the parity (exact) mode and in the fast mode: <= 1e-10 relative L2 on U, V, Ux, Uy,
  with the same Picard count and the same number of SOR sweeps in every linear solve;
* mixed precision (FP32 correction sweeps in FP64 defect correction): <= 1e-6 relative L2.

Everything is built by the oracle (mesh, neighbour functions, colouring, geometry), so the
inputs cannot share a defect with the library's own host code.
"""
import os

import numpy as np
import pytest

from conftest import oracle_aaac, oracle_inputs, rel_l2

import oracle as orc
from ufemism_gb300 import _native as nat
from ufemism_gb300 import api

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6
FIELDS = ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac")


@pytest.fixture(scope="module")
def dome200k():
    api.init(0)
    m = oracle_aaac("200k")
    ssa, sia, g = oracle_inputs(m)
    rc, out, st = orc.solve_ssa(m, ssa, orc.default_params(n_threads=os.cpu_count() or 1))
    # From the cold start the first linear solve stops at the reference's 10,000-sweep cap
    # (the reference's non-convergence warning, UFE_NOT_CONVERGED); the later ones converge.
    assert rc in (orc.OR_OK, orc.OR_NOT_CONVERGED), rc
    out["status"] = rc
    dm = api.DeviceMesh(m)
    yield m, ssa, (out, st), dm
    dm.close()


def _errors(gout, oout):
    return {k: rel_l2(gout[k], oout[k]) for k in FIELDS}


@pytest.mark.parametrize("exact", [1, 0])
def test_200k_fp64_matches_oracle(dome200k, exact):
    m, ssa, (oout, ost), dm = dome200k
    rc, gout, gst = dm.solve_ssa(ssa, api.default_params(precision=nat.UFE_FP64, fp64_exact=exact), check=False)
    assert rc == oout["status"]
    assert gst["picard_iterations"] == ost["picard_iterations"]
    assert gst["sweeps"] == ost["sweeps"], (gst["sweeps"], ost["sweeps"])
    err = _errors(gout, oout)
    assert max(err.values()) <= FP64_TOL, err
    for k in ("N_AaAc", "Up_SSA_Ac", "Uo_SSA_Ac"):
        assert rel_l2(gout[k], oout[k]) <= FP64_TOL, k


def test_200k_mixed_matches_oracle(dome200k):
    m, ssa, (oout, ost), dm = dome200k
    rc, gout, gst = dm.solve_ssa(ssa, api.default_params(precision=nat.UFE_MIXED), check=False)
    assert rc == oout["status"]
    assert gst["sweeps"][0] == ost["sweeps"][0]   # the capped first linear solve
    assert gst["picard_iterations"] == ost["picard_iterations"]
    err = _errors(gout, oout)
    assert max(err.values()) <= MIXED_TOL, err
    # the dome flows outwards between the summit and the margin
    x, y = m.base.V[:, 0], m.base.V[:, 1]
    r = np.hypot(x, y)
    sel = (r > 200e3) & (r < 600e3)
    ur = (gout["U_SSA"][sel] * x[sel] + gout["V_SSA"][sel] * y[sel]) / r[sel]
    assert np.all(ur > 0)


@pytest.mark.parametrize("precision", [nat.UFE_FP64, nat.UFE_MIXED])
def test_200k_phased_sweeps_match_oracle(dome200k, monkeypatch, precision):
    """The phased sweeps (one grid-wide phase per colour; the path of the batched members),
    selected for a single solve with UFE_SSA_HALO=0, against the same oracle result."""
    m, ssa, (oout, ost), dm = dome200k
    monkeypatch.setenv("UFE_SSA_HALO", "0")
    rc, gout, gst = dm.solve_ssa(ssa, api.default_params(precision=precision, fp64_exact=0), check=False)
    assert rc == oout["status"]
    assert gst["picard_iterations"] == ost["picard_iterations"]
    err = _errors(gout, oout)
    if precision == nat.UFE_FP64:
        assert gst["sweeps"] == ost["sweeps"]
        assert max(err.values()) <= FP64_TOL, err
    else:
        assert gst["sweeps"][0] == ost["sweeps"][0]
        assert max(err.values()) <= MIXED_TOL, err


@pytest.fixture(scope="module")
def marine16k():
    """The marine setup (sloping bed with a Gaussian random field, floating shelf) on a 16k
    mesh: the largest of the seeded marine meshes on which the reference's SOR converges
    within its 10,000-sweep cap after the cold-start linear solve (from 50k vertices up,
    every linear solve of the oracle stops at the cap)."""
    api.init(0)
    m = oracle_aaac("16k")
    ssa, sia, g = oracle_inputs(m, "marine")
    assert g["mask_shelf"].sum() > 0
    rc, out, st = orc.solve_ssa(m, ssa, orc.default_params(n_threads=os.cpu_count() or 1))
    assert rc in (orc.OR_OK, orc.OR_NOT_CONVERGED), rc
    assert all(s < 10000 for s in st["sweeps"][1:]), st["sweeps"]
    out["status"] = rc
    dm = api.DeviceMesh(m)
    yield m, ssa, (out, st), dm
    dm.close()


def test_16k_marine_fp64_and_mixed_match_oracle(marine16k):
    m, ssa, (oout, ost), dm = marine16k
    rc, gout, gst = dm.solve_ssa(ssa, api.default_params(precision=nat.UFE_FP64), check=False)
    assert rc == oout["status"]
    assert gst["sweeps"] == ost["sweeps"]
    assert max(_errors(gout, oout).values()) <= FP64_TOL
    rc, gout, gst = dm.solve_ssa(ssa, api.default_params(precision=nat.UFE_MIXED), check=False)
    assert rc == oout["status"]
    assert gst["picard_iterations"] == ost["picard_iterations"]
    err = _errors(gout, oout)
    assert max(err.values()) <= MIXED_TOL, err
