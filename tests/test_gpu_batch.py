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
        assert timing["max_team_ctas"] == 4 and timing["n_classes"] == 1
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


@pytest.mark.parametrize("block,team,rows,graph", [(512, 2, 0, True), (256, 8, 0, True), (1024, 1, 0, False),
                                                   (1024, 0, 4096, True), (256, 0, 2048, True)])
def test_batch_shapes(ensemble, block, team, rows, graph):
    """Uniform teams (team > 0) and per-member team sizes from a rows-per-CTA packing."""
    single = single_results(ensemble, nat.UFE_MIXED)
    b, p, rc, stats, timing, outs = run_batch(ensemble, nat.UFE_MIXED, team_ctas=team, rows_per_cta=rows,
                                              block=block, use_graph=graph)
    try:
        assert rc >= 0
        assert timing["block"] == block
        if team:
            assert timing["max_team_ctas"] == team and timing["n_classes"] == 1
        else:
            assert timing["n_classes"] >= 2
        check_members(single, stats, outs)
    finally:
        b.close()


def test_solve_batched_one_call(ensemble):
    """ufe_ssa_solve_batched (create, upload, run, download, destroy in one call)."""
    import ctypes as ct
    single = single_results(ensemble, nat.UFE_MIXED)
    L = nat.load()
    n = len(ensemble)
    descs = (nat.MeshDesc * n)()
    ins = (nat.SsaIn * n)()
    ios = (nat.SsaInout * n)()
    keep = []
    outs = []
    for i, (base, mesh, ssa) in enumerate(ensemble):
        d, k = api._mesh_desc(mesh)
        descs[i] = d
        si, sio, io, kk = api._ssa_structs(base.nV, mesh.nAc, mesh.nVAaAc, ssa, None)
        ins[i] = si
        ios[i] = sio
        keep += [k, kk]
        outs.append(io)
    p = api.default_params(precision=nat.UFE_MIXED)
    ps, _z = api._params_struct(p)
    st = (nat.SsaStats * n)()
    cfg = nat.BatchConfig(0, 4096, 0, 1)
    rc = L.ufe_ssa_solve_batched(n, descs, ct.byref(cfg), ct.byref(ps), ins, ios, None, st)
    assert rc >= 0, nat.last_error()
    check_members(single, [api.stats_dict(x) for x in st], outs)


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


def test_autotune_picks_a_tried_candidate(ensemble):
    p = api.default_params(precision=nat.UFE_MIXED)
    best, tried = api.batch_autotune(ensemble, p)
    assert len(tried) >= 3
    fastest = min(tried, key=lambda e: e["device_ms"])
    assert (best["rows_per_cta"], best["block"]) == (fastest["rows_per_cta"], fastest["block"])
    assert all(e["device_ms"] > 0 for e in tried)


def test_batch_with_early_out_member_and_coulomb_gl_members():
    """A member without grounded ice takes the early-out (zero velocities, not queued); the
    Coulomb law with the grounding-line flux rows runs batched exactly as single solves."""
    from conftest import oracle_aaac, oracle_inputs
    api.init(0)
    m1 = oracle_aaac("1k")
    ssa_m, _, _ = oracle_inputs(m1, "marine")
    ssa_d, _, _ = oracle_inputs(m1, "dome")
    empty = dict(ssa_d, Hi=np.zeros_like(ssa_d["Hi"]), mask_sheet=np.zeros_like(ssa_d["mask_sheet"]))
    p = api.default_params(precision=nat.UFE_MIXED, sliding_law=nat.UFE_SLIDING_COULOMB_REGULARISED,
                           use_analytical_GL_flux=1)
    members = [ssa_m, empty, ssa_m, ssa_d]
    single = []
    for f in members:
        dm = api.DeviceMesh(m1)
        single.append(dm.solve_ssa(f, p, check=False))
        dm.close()
    b = api.Batch([m1] * len(members), rows_per_cta=2048)
    try:
        for i, f in enumerate(members):
            b.upload(i, f, p)
        rc, stats, timing = b.run(p, check=False)
        assert timing["n_active"] == len(members) - 1
        outs = [b.download(i) for i in range(b.n)]
        assert np.all(outs[1]["U_SSA"] == 0.0) and np.all(outs[1]["Ux_SSA_Ac"] == 0.0)
        for i in (0, 2, 3):
            rc1, o1, s1 = single[i]
            assert stats[i]["sweeps"] == s1["sweeps"], i
            for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac"):
                assert rel_l2(outs[i][k], o1[k]) <= TOL, (i, k)
    finally:
        b.close()


def test_batch_into_reused_host_buffers(ensemble):
    """upload/download with per-member host buffers (warm start read in place, results written
    in place) give the members' single solves, twice from a reset of the same arrays."""
    single = single_results(ensemble, nat.UFE_MIXED)
    b = api.Batch([m for _, m, _ in ensemble])
    p = api.default_params(precision=nat.UFE_MIXED, sliding_law=nat.UFE_SLIDING_LINEAR)
    bufs = [api.ssa_buffers(base.nV, mesh.nAc, mesh.nVAaAc) for base, mesh, _ in ensemble]
    for _ in range(2):
        for i, (_, _, ssa) in enumerate(ensemble):
            for k in api.SSA_INOUT_FIELDS:
                bufs[i][k].fill(0.0)
            b.upload(i, ssa, p, buffers=bufs[i])
        rc, stats, timing = b.run(p)
        outs = [b.download(i, buffers=bufs[i]) for i in range(b.n)]
        assert all(o is bb for o, bb in zip(outs, bufs))
        check_members(single, stats, outs)
    b.close()


ORACLE_SIZES = (2200, 5200, 12000)   # config-4 style members: GRF friction, H0 drawn per member


@pytest.fixture(scope="module")
def oracle_members():
    """Three ensemble members (log-uniform sizes, dome H0 from U[2000, 4000] m, log beta^2 a
    Gaussian random field with std 1 and 100 km correlation), each with the oracle's FP64
    solve on a mesh the oracle built itself."""
    import os
    import oracle as orc
    api.init(0)
    out = []
    for i, n in enumerate(ORACLE_SIZES):
        base, mesh, ssa = wl.ensemble_member(n, 9100 + i)
        om = orc.build_aaac(base)
        for k in ("CAaAc", "colour_vi", "Nxx_AaAc"):
            assert np.array_equal(np.asarray(getattr(om, k)), np.asarray(getattr(mesh, k))), k
        rc, oo, st = orc.solve_ssa(om, ssa, orc.default_params(n_threads=os.cpu_count() or 1))
        assert rc in (orc.OR_OK, orc.OR_NOT_CONVERGED)
        st["status"] = rc
        out.append((base, mesh, ssa, oo, st))
    return out


@pytest.mark.parametrize("precision", [nat.UFE_FP64, nat.UFE_MIXED])
def test_batch_members_match_oracle(oracle_members, precision):
    """Batched members against the oracle directly (not only against the library's single
    solves): FP64 <= 1e-10 with the oracle's Picard and sweep counts, mixed <= 1e-6."""
    ens = [(b, m, s) for b, m, s, _, _ in oracle_members]
    bt, p, rc, stats, timing, outs = run_batch(ens, precision, rows_per_cta=2048)
    try:
        assert rc >= 0
        for i, (_, _, _, oo, ost) in enumerate(oracle_members):
            assert stats[i]["status"] == ost["status"], i
            assert stats[i]["picard_iterations"] == ost["picard_iterations"], i
            if precision == nat.UFE_FP64:
                assert stats[i]["sweeps"] == ost["sweeps"], i
            tol = 1e-10 if precision == nat.UFE_FP64 else 1e-6
            for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac"):
                assert rel_l2(outs[i][k], oo[k]) <= tol, (i, k, rel_l2(outs[i][k], oo[k]))
    finally:
        bt.close()
