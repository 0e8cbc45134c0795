"""GPU SSA/SIA solve through the C-ABI against the CPU oracle (run with -m gpu).

Tolerances: FP64 path <= 1e-10 relative L2 on u and v with identical Picard and SOR
iteration counts; mixed path <= 1e-6 relative L2; SIA <= 1e-12.
"""
import numpy as np
import pytest

from conftest import base_mesh, oracle_aaac, oracle_inputs, rel_l2

import oracle as orc
from ufemism_gb300 import _native as nat
from ufemism_gb300 import api

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def device():
    api.init(0)   # raises (fails the test) without a usable sm_103a device
    yield


_DEV = {}


def device_mesh(name):
    if name not in _DEV:
        _DEV[name] = api.DeviceMesh(oracle_aaac(name))
    return _DEV[name]


def oracle_params(**kw):
    return orc.default_params(**kw)


def gpu_params(**kw):
    p = api.default_params(**{k: v for k, v in kw.items() if k in api.default_params()})
    return p


def _check_solution(gout, oout, tol):
    for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac"):
        e = rel_l2(gout[k], oout[k])
        assert e <= tol, "%s rel-L2 %.3e > %.1e" % (k, e, tol)


def _run_both(name, kind="dome", precision=nat.UFE_FP64, warm=None, oracle_kw=None, gpu_kw=None, fields_kw=None):
    m = oracle_aaac(name)
    ssa, sia, g = oracle_inputs(m, kind)
    if fields_kw:
        ssa.update(fields_kw)
    okw = dict(oracle_kw or {})
    gkw = dict(gpu_kw or {})
    rc_o, oout, ost = orc.solve_ssa(m, dict(ssa, **(warm or {})), oracle_params(**okw))
    gp = api.default_params(precision=precision, **gkw)
    rc_g, gout, gst = device_mesh(name).solve_ssa(ssa, gp, warm=warm, check=False)
    return m, (rc_o, oout, ost), (rc_g, gout, gst)


@pytest.mark.parametrize("exact", [0, 1])
@pytest.mark.parametrize("name", ["tiny", "1k", "4k"])
def test_fp64_dome_linear_matches_oracle(name, exact):
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both(name, gpu_kw=dict(fp64_exact=exact))
    assert rc_g == rc_o == 0
    assert gst["picard_iterations"] == ost["picard_iterations"]
    assert gst["sweeps"] == ost["sweeps"]
    _check_solution(gout, oout, FP64_TOL)
    for k in ("N_AaAc", "eta_AaAc", "Up_SSA_Ac", "Uo_SSA_Ac"):
        assert rel_l2(gout[k], oout[k]) <= FP64_TOL, k


def test_fp64_coulomb_law_matches_oracle():
    kw = dict(sliding_law=nat.UFE_SLIDING_COULOMB_REGULARISED)
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("1k", oracle_kw=dict(sliding_law=0), gpu_kw=kw)
    assert rc_g == rc_o
    assert gst["sweeps"] == ost["sweeps"]
    _check_solution(gout, oout, FP64_TOL)
    for k in ("tau_c_AaAc", "phi_fric_AaAc", "S_AaAc"):
        assert rel_l2(gout[k], oout[k]) <= FP64_TOL, k


def test_fp64_marine_beta_field_matches_oracle():
    m = oracle_aaac("4k")
    from ufemism_gb300 import workloads as wl
    beta = np.exp(wl.log_beta_field(m, std=1.0, ell=100e3, seed=5))
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("4k", kind="marine", fields_kw=dict(beta_sq_AaAc=beta))
    ssa, sia, g = oracle_inputs(m, "marine")
    assert g["mask_shelf"].sum() > 0, "marine case must have floating ice"
    assert rc_g == rc_o
    assert gst["sweeps"] == ost["sweeps"]
    _check_solution(gout, oout, FP64_TOL)


def test_fp64_gl_flux_matches_oracle():
    kw = dict(sliding_law=0, use_analytical_GL_flux=1)
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("4k", kind="marine", oracle_kw=kw, gpu_kw=kw)
    ssa, sia, g = oracle_inputs(m, "marine")
    assert g["mask_gl_Ac"].sum() > 0
    assert rc_g == rc_o
    assert gst["sweeps"] == ost["sweeps"]
    _check_solution(gout, oout, FP64_TOL)


def test_fp64_warm_start_and_picard_state():
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("1k")
    warm_o = {k: oout[k] for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "N_AaAc")}
    warm_g = {k: gout[k] for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "N_AaAc")}
    ssa, sia, g = oracle_inputs(m)
    rc_o2, oout2, ost2 = orc.solve_ssa(m, dict(ssa, **warm_o), oracle_params())
    rc_g2, gout2, gst2 = device_mesh("1k").solve_ssa(ssa, api.default_params(), warm=warm_g)
    assert gst2["picard_iterations"] == ost2["picard_iterations"]
    assert gst2["sweeps"] == ost2["sweeps"]
    _check_solution(gout2, oout2, FP64_TOL)


@pytest.mark.parametrize("name", ["1k", "4k"])
def test_mixed_matches_oracle(name):
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both(name, precision=nat.UFE_MIXED)
    assert rc_g == rc_o == 0
    _check_solution(gout, oout, MIXED_TOL)
    # same discrete trajectory: the Picard count is the FP64 one
    assert gst["picard_iterations"] == ost["picard_iterations"]


def test_mixed_fp32_viscosity_dome():
    """The mixed form with the viscosity in FP32 as well (FP32 arithmetic on FP64 velocity
    differences): within 1e-6 on the grounded dome. On the marine case the FP32 viscosity
    alone gives 1.3e-6, which is why the viscosity defaults to FP64 in the mixed path."""
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("4k", precision=nat.UFE_MIXED,
                                                        gpu_kw=dict(mixed_fp32_viscosity=1))
    assert rc_g == rc_o == 0
    _check_solution(gout, oout, MIXED_TOL)


def test_mixed_marine_matches_oracle():
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("4k", kind="marine", precision=nat.UFE_MIXED)
    assert rc_g == rc_o
    _check_solution(gout, oout, MIXED_TOL)


def test_reset_once_then_converged_like_reference():
    """omega = 2.5 makes SOR diverge: the residual passes 1e6, velocities are reset to zero
    (ice_dynamics_module.f90:679-684); from the cold start the next viscosity equals the
    previous one, RN = 0 and the solve ends with one reset (UFE_RESET_ONCE)."""
    kw = dict(SSA_SOR_omega=2.5)
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("tiny", oracle_kw=kw, gpu_kw=kw)
    assert rc_o == orc.OR_RESET_ONCE and rc_g == nat.UFE_RESET_ONCE
    assert gst["resets"] == ost["resets"] == 1
    assert gst["sweeps"] == ost["sweeps"]
    assert np.all(gout["U_SSA"] == 0.0)


def test_second_reset_is_divergence_like_reference():
    """Warm-started velocities without the Picard state: the first linear solve diverges and
    resets, the viscosity then changes, the second linear solve diverges too: the reference
    aborts (532-540), the library returns UFE_DIVERGED."""
    m = oracle_aaac("tiny")
    ssa, sia, g = oracle_inputs(m)
    rc0, out0, st0 = orc.solve_ssa(m, ssa, oracle_params())
    warm = {k: out0[k] for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac")}
    rc_o, oout, ost = orc.solve_ssa(m, dict(ssa, **warm), oracle_params(SSA_SOR_omega=2.5))
    rc_g, gout, gst = device_mesh("tiny").solve_ssa(ssa, api.default_params(SSA_SOR_omega=2.5), warm=warm,
                                                    check=False)
    assert rc_o == orc.OR_ERR_DIVERGED
    assert rc_g == nat.UFE_DIVERGED
    assert gst["resets"] == ost["resets"] == 2
    assert gst["sweeps"] == ost["sweeps"]


def test_not_converged_warning():
    kw = dict(SSA_max_inner_loops=20, SSA_max_outer_loops=3)
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("1k", oracle_kw=kw, gpu_kw=kw)
    assert rc_o == orc.OR_NOT_CONVERGED and rc_g == nat.UFE_NOT_CONVERGED
    assert gst["sweeps"] == ost["sweeps"] and ost["sweeps"][0] == 20
    _check_solution(gout, oout, FP64_TOL)


MIXED_LAG = 1   # the mixed sweeps decide convergence this many sweeps late (ufe_ssa.cu, kMixedLag)


def test_mixed_lagged_decisions_cap_and_reset():
    """The mixed sweeps decide convergence from the residual of the sweep `MIXED_LAG` earlier,
    with no team barrier between sweeps, and decide exactly at the sweep cap: a capped solve
    stops at the cap and warns like the reference, a converged one has done at least
    MIXED_LAG + 1 sweeps and ends below the tolerance, and a diverging one resets once."""
    kw = dict(SSA_max_inner_loops=20, SSA_max_outer_loops=3)
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("1k", precision=nat.UFE_MIXED, oracle_kw=kw, gpu_kw=kw)
    assert rc_o == orc.OR_NOT_CONVERGED and rc_g == nat.UFE_NOT_CONVERGED
    assert gst["sweeps"][0] == 20 and all(sw <= 20 for sw in gst["sweeps"])
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("4k", precision=nat.UFE_MIXED,
                                                        gpu_kw=dict(mixed_refold_sweeps=8))
    assert rc_g == rc_o == 0
    _check_solution(gout, oout, MIXED_TOL)
    assert all(sw >= MIXED_LAG + 1 for sw in gst["sweeps"])
    assert gst["last_max_residual"] < api.default_params()["SSA_max_residual_UV"]
    kw = dict(SSA_SOR_omega=2.5)
    m, (rc_o, oout, ost), (rc_g, gout, gst) = _run_both("tiny", precision=nat.UFE_MIXED, oracle_kw=kw, gpu_kw=kw)
    assert rc_o == orc.OR_RESET_ONCE and rc_g == nat.UFE_RESET_ONCE
    assert gst["resets"] == 1 and np.all(gout["U_SSA"] == 0.0)


def test_early_outs_zero_velocity():
    m = oracle_aaac("tiny")
    ssa, sia, g = oracle_inputs(m)
    warm = dict(U_SSA=np.ones(m.base.nV), V_SSA=np.ones(m.base.nV), Ux_SSA_Ac=np.ones(m.nAc),
                Uy_SSA_Ac=np.ones(m.nAc))
    rc, out, st = device_mesh("tiny").solve_ssa(ssa, api.default_params(zero_velocities=1), warm=warm)
    assert rc == 0 and st["picard_iterations"] == 0
    for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "Up_SSA_Ac", "Uo_SSA_Ac"):
        assert np.all(out[k] == 0.0), k
    no_ice = dict(ssa, mask_sheet=np.zeros(m.base.nV, dtype=np.int32))
    rc, out, st = device_mesh("tiny").solve_ssa(no_ice, api.default_params(), warm=warm)
    assert rc == 0 and np.all(out["U_SSA"] == 0.0)


def test_split_entry_points_repeatable():
    """ufe_ssa_upload once, ufe_ssa_run twice on the same device-resident inputs."""
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m)
    dm = device_mesh("1k")
    p = api.default_params()
    dm.ssa_upload(ssa, p)
    rc1, st1 = dm.ssa_run(p)
    o1 = dm.ssa_download()
    rc2, st2 = dm.ssa_run(p)
    o2 = dm.ssa_download()
    assert st1["sweeps"] == st2["sweeps"]
    assert np.array_equal(o1["U_SSA"], o2["U_SSA"])


@pytest.mark.parametrize("name", ["1k", "4k"])
def test_sia_matches_oracle(name):
    m = oracle_aaac(name)
    ssa, sia, g = oracle_inputs(m)
    oo = orc.solve_sia(m, sia, orc.default_params())
    go = device_mesh(name).solve_sia(sia, api.default_params())
    for k in ("D_SIA_3D_Ac", "D_SIA_Ac", "Ux_SIA_Ac", "Uy_SIA_Ac", "Up_SIA_Ac", "Uo_SIA_Ac", "U_SIA", "V_SIA",
              "D_SIA"):
        assert rel_l2(go[k], oo[k]) <= 1e-12, k


def test_solve_into_reused_host_buffers():
    """solve_ssa(buffers=...) reads the warm start from the caller's arrays and writes every
    result into them in place; the same solve as the allocating form, repeated from a reset."""
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m)
    dm = device_mesh("1k")
    p = api.default_params(precision=nat.UFE_MIXED)
    rc1, o1, s1 = dm.solve_ssa(ssa, p)
    bufs = dm.ssa_buffers()
    keep = {k: bufs[k] for k in bufs}
    for _ in range(2):
        for k in api.SSA_INOUT_FIELDS:
            bufs[k].fill(0.0)
        rc2, o2, s2 = dm.solve_ssa(ssa, p, buffers=bufs)
        assert rc2 == rc1 and s2["sweeps"] == s1["sweeps"]
        for k in api.SSA_INOUT_FIELDS + api.SSA_OUT_FIELDS:
            assert o2[k] is keep[k] and np.array_equal(o2[k], o1[k]), k
    with pytest.raises(ValueError):
        dm.solve_ssa(ssa, p, buffers=dict(bufs, U_SSA=np.zeros(3)))
