"""Batched ensemble solve through the C-ABI (run with -m gpu).

Every member of a batch must give the solution of the same problem solved alone through
ufe_ssa_solve: the sweeps of one colour are independent, so the patch layout changes no
arithmetic, and only the order of the RN partial sums differs (it could flip a Picard
decision only if RN landed within rounding of the tolerance). Tolerance 1e-12 relative L2,
with identical Picard and SOR iteration counts.
"""
import numpy as np
import pytest

from conftest import rel_l2

from ufemism_gb300 import _native as nat
from ufemism_gb300 import api
from ufemism_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-12
SIZES = (1500, 4200, 2300, 6000, 3100, 1800)


@pytest.fixture(scope="module")
def ensemble():
    api.init(0)
    return [wl.ensemble_member(n, 7000 + i) for i, n in enumerate(SIZES)]


_SINGLE = {}


def single_results(ensemble, precision, exact=0):
    key = (precision, exact)
    if key not in _SINGLE:
        res = []
        for base, mesh, ssa in ensemble:
            dm = api.DeviceMesh(mesh)
            p = api.default_params(precision=precision, fp64_exact=exact, sliding_law=nat.UFE_SLIDING_LINEAR)
            rc, out, st = dm.solve_ssa(ssa, p)
            dm.close()
            res.append((rc, out, st))
        _SINGLE[key] = res
    return _SINGLE[key]


def run_batch(ensemble, precision, exact=0, **cfg):
    b = api.Batch([m for _, m, _ in ensemble], **cfg)
    p = api.default_params(precision=precision, fp64_exact=exact, sliding_law=nat.UFE_SLIDING_LINEAR)
    for i, (_, _, ssa) in enumerate(ensemble):
        b.upload(i, ssa, p)
    rc, stats, timing = b.run(p)
    outs = [b.download(i) for i in range(b.n)]
    return b, p, rc, stats, timing, outs


def check_members(single, stats, outs):
    for i, ((rc1, o1, s1), s2, o2) in enumerate(zip(single, stats, outs)):
        assert s2["status"] == rc1, i
        assert s2["picard_iterations"] == s1["picard_iterations"], i
        assert s2["sweeps"] == s1["sweeps"], i
        for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac"):
            assert rel_l2(o2[k], o1[k]) <= TOL, (i, k)


@pytest.mark.parametrize("precision", [nat.UFE_MIXED, nat.UFE_FP64])
def test_batch_matches_single_solves(ensemble, precision):
    single = single_results(ensemble, precision)
    b, p, rc, stats, timing, outs = run_batch(ensemble, precision, team_ctas=4)
    try:
        assert rc >= 0
        check_members(single, stats, outs)
        assert timing["n_active"] == len(ensemble)
        assert timing["team_ctas"] == 4
        assert 0 < timing["member_p50_ms"] <= timing["member_p99_ms"] <= timing["member_max_ms"]
        assert np.all(timing["member_ms"] > 0)
        # graph replay: the same results again
        rc2, stats2, timing2 = b.run(p)
        assert rc2 == rc
        for i in range(b.n):
            assert stats2[i]["sweeps"] == stats[i]["sweeps"]
            assert np.array_equal(b.download(i)["U_SSA"], outs[i]["U_SSA"])
    finally:
        b.close()


@pytest.mark.parametrize("block,team,graph", [(512, 2, True), (256, 8, True), (1024, 1, False)])
def test_batch_shapes(ensemble, block, team, graph):
    single = single_results(ensemble, nat.UFE_MIXED)
    b, p, rc, stats, timing, outs = run_batch(ensemble, nat.UFE_MIXED, team_ctas=team, block=block,
                                              use_graph=graph)
    try:
        assert rc >= 0
        assert timing["block"] == block and timing["team_ctas"] == team
        check_members(single, stats, outs)
    finally:
        b.close()


def test_batch_exact_fp64_bitwise(ensemble):
    single = single_results(ensemble, nat.UFE_FP64, exact=1)
    b, p, rc, stats, timing, outs = run_batch(ensemble, nat.UFE_FP64, exact=1, team_ctas=3)
    try:
        check_members(single, stats, outs)
    finally:
        b.close()


def test_batch_rejects_team_larger_than_member(ensemble):
    with pytest.raises(nat.UfeError) as e:
        api.Batch([ensemble[0][1]], team_ctas=400)
    assert e.value.status in (nat.UFE_BAD_ARG, nat.UFE_BAD_MESH)
