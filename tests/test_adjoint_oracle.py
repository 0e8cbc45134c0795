"""The FP64 CPU adjoint reference (oracle/ssa_adjoint.py) pinned against the oracle's own
forward solve: its Jacobian against finite differences of the residual, and its gradients
against central finite differences of the misfit (h = 1e-4) and against its tangent-linear
model. Runs on CPU."""
import numpy as np
import pytest

from conftest import oracle_aaac, oracle_inputs

import oracle as orc
import ssa_adjoint as adj
from ufemism_gb300 import workloads as wl

TIGHT = dict(SSA_RN_tol=1e-13, SSA_max_residual_UV=1e-11, SSA_max_outer_loops=300, SSA_max_inner_loops=1000000)


@pytest.fixture(scope="module")
def problem():
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m, "dome")
    logb = wl.log_beta_field(m, std=1.0, ell=100e3, seed=5)
    P = orc.default_params(**TIGHT)

    def solve(lb, fields=None):
        f = dict(fields or ssa)
        f["beta_sq_AaAc"] = np.exp(lb)
        rc, out, st = orc.solve_ssa(m, f, P)
        assert rc == 0 and st["last_RN"] < 1e-12
        return adj.aaac_velocity(out), f

    (U, V), f0 = solve(logb)
    (Uo, Vo), _ = solve(logb + wl.log_beta_field(m, std=0.3, ell=100e3, seed=11))
    return m, ssa, logb, solve, U, V, f0, Uo, Vo


def fields_for(m, ssa, H):
    g = orc.update_geometry(m, H, ssa["Hb"], ssa["SL"])
    f = dict(ssa)
    for k in ("Hi_Ac", "dHs_dx_shelf", "dHs_dy_shelf", "dHs_dx_shelf_Ac", "dHs_dy_shelf_Ac", "Hb_Ac", "SL_Ac"):
        f[k] = g[k]
    f["Hi"] = H
    return f, g


def test_residual_vanishes_and_jacobian_matches_finite_differences(problem):
    m, ssa, logb, solve, U, V, f0, Uo, Vo = problem
    lin = adj.Linearisation(m, f0, U, V)
    F = lin.residual()
    scale = np.abs(adj.RHO_I * adj.GRAV * lin.g["hx"] / lin.eta).max()    # driving-stress term
    assert np.abs(F).max() < 1e-9 * scale
    K = lin.jacobian()
    rng = np.random.default_rng(0)
    nA = m.nVAaAc
    for _ in range(2):
        d = rng.normal(size=2 * nA)
        h = 1e-6 * np.abs(U).max()
        Fp = adj.Linearisation(m, f0, U + h * d[:nA], V + h * d[nA:]).residual()
        Fm = adj.Linearisation(m, f0, U - h * d[:nA], V - h * d[nA:]).residual()
        fd = (Fp - Fm) / (2 * h)
        an = K @ d
        assert np.linalg.norm(fd - an) / np.linalg.norm(an) < 1e-7


def test_gradients_match_finite_differences_and_tangent_linear(problem):
    m, ssa, logb, solve, U, V, f0, Uo, Vo = problem
    lin = adj.Linearisation(m, f0, U, V)
    G = adj.geometry_matrix(m, ssa["Hi"], ssa["Hb"], ssa["SL"])
    gU, gV = U - Uo, V - Vo
    mx, my, dlb, dHi, sens = adj.adjoint_gradient(lin, gU, gV, G)
    rng = np.random.default_rng(1)
    h = 1e-4
    for _ in range(2):
        d = rng.normal(size=m.nVAaAc)
        (Up, Vp), _ = solve(logb + h * d)
        (Um, Vm), _ = solve(logb - h * d)
        fd = (adj.misfit(Up, Vp, Uo, Vo) - adj.misfit(Um, Vm, Uo, Vo)) / (2 * h)
        an = float(dlb @ d)
        du, dv = adj.tangent_linear(lin, d_logbeta=d)
        assert abs(fd - an) <= 1e-5 * abs(an)
        assert abs(float(gU @ du + gV @ dv) - an) <= 1e-10 * abs(an)
    Hi = ssa["Hi"]
    for _ in range(2):
        d = rng.normal(size=m.base.nV) * (Hi > 50.0)
        fp, gp = fields_for(m, ssa, Hi + h * d)
        fm, gm = fields_for(m, ssa, Hi - h * d)
        assert np.array_equal(gp["mask_ocean"], gm["mask_ocean"])
        (Up, Vp), _ = solve(logb, fp)
        (Um, Vm), _ = solve(logb, fm)
        fd = (adj.misfit(Up, Vp, Uo, Vo) - adj.misfit(Um, Vm, Uo, Vo)) / (2 * h)
        an = float(dHi @ d)
        du, dv = adj.tangent_linear(lin, d_Hi=d, G=G)
        assert abs(fd - an) <= 1e-5 * abs(an)
        assert abs(float(gU @ du + gV @ dv) - an) <= 1e-10 * abs(an)


@pytest.fixture(scope="module")
def coulomb():
    """The marine 1k case under the reference's Coulomb_regularised law (floating shelf rows
    without friction), solved tightly by the oracle."""
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m, "marine")
    P = orc.default_params(sliding_law=0, **TIGHT)

    def solve(fields):
        rc, out, st = orc.solve_ssa(m, fields, P)
        assert rc == 0 and st["last_RN"] < 1e-12
        return adj.aaac_velocity(out), out

    (U, V), out = solve(ssa)
    return m, ssa, solve, U, V, out


def test_coulomb_jacobian_matches_finite_differences(coulomb):
    """With the velocity-dependent sliding term S(u) of the Coulomb law, the residual vanishes at
    the oracle's converged state and the Jacobian, S'(u) blocks included, matches central finite
    differences of the residual. The direction lives on the grounded interior rows, scaled by
    each row's speed plus the regularisation dv (grounded rows here run as slow as 4e-5 m/yr,
    below dv = 1e-3, where a uniform step would see S's curvature); on it the S'(u) blocks carry
    a third of the Jacobian's action, so leaving them out fails the comparison."""
    m, ssa, solve, U, V, out = coulomb
    tau = out["tau_c_AaAc"]
    lin = adj.Linearisation(m, ssa, U, V, tau_c=tau)
    F = lin.residual()
    interior = np.concatenate([~lin.edge, ~lin.edge])
    scale = np.abs(adj.RHO_I * adj.GRAV * lin.g["hx"] / lin.eta).max()
    assert np.abs(F[interior]).max() < 1e-9 * scale                      # momentum rows
    assert np.abs(F[~interior]).max() < 1e-12 * np.abs(np.concatenate([U, V])).max()   # Neumann rows
    assert np.any(lin.fr > 0) and np.any(lin.floating & ~lin.edge)
    K = lin.jacobian()
    nA = m.nVAaAc
    rng = np.random.default_rng(3)
    grounded = np.concatenate([lin.fr > 0, lin.fr > 0])
    speed = np.hypot(U, V) + adj.DELTA_V
    h = 1e-5
    for _ in range(2):
        d = np.where(grounded, np.concatenate([speed, speed]) * rng.normal(size=2 * nA), 0.0)
        Fp = adj.Linearisation(m, ssa, U + h * d[:nA], V + h * d[nA:], tau_c=tau).residual()
        Fm = adj.Linearisation(m, ssa, U - h * d[:nA], V - h * d[nA:], tau_c=tau).residual()
        an = K @ d
        assert np.linalg.norm((Fp - Fm) / (2 * h) - an) / np.linalg.norm(an) < 1e-8
    # the same friction factor treated as a constant of u (no S'(u) blocks)
    frozen = adj.Linearisation(m, ssa, U, V, tau_c=tau)
    frozen.tau_c = None
    frozen.g = dict(frozen.g, beta=tau * lin.w ** (0.5 * (adj.Q_PLASTIC - 1.0)) / adj.U_THRESHOLD ** adj.Q_PLASTIC)
    frozen.update(U, V)
    assert np.linalg.norm((frozen.jacobian() - K) @ d) > 0.1 * np.linalg.norm(K @ d)


def test_coulomb_thickness_gradient_matches_finite_differences(coulomb):
    """dJ/dHi under the Coulomb law against central finite differences of the oracle's forward
    solve, on perturbations away from the floatation and ice-free thresholds (masks frozen)."""
    m, ssa, solve, U, V, out = coulomb
    H = np.asarray(ssa["Hi"], dtype=np.float64)
    Hb, SL = ssa["Hb"], ssa["SL"]
    rng = np.random.default_rng(12)
    x, y = m.base.V[:, 0], m.base.V[:, 1]
    bump = 20.0 * np.exp(-((x - 2e5) ** 2 + (y + 1e5) ** 2) / (2 * (1.5e5) ** 2))
    (Uo, Vo), _ = solve(fields_for(m, ssa, np.where(H > 0, H + bump, H))[0])
    lin = adj.Linearisation(m, ssa, U, V, tau_c=out["tau_c_AaAc"])
    G = adj.geometry_matrix(m, H, Hb, SL)
    gU, gV = U - Uo, V - Vo
    mx, my, dlb, dHi, sens = adj.adjoint_gradient(lin, gU, gV, G)
    flot = (SL - Hb) * adj.RHO_SW / adj.RHO_I
    safe = (H > 50.0) & (np.abs(H - flot) > 50.0)
    h = 1e-2
    for _ in range(2):
        d = np.where(safe, rng.normal(size=H.size), 0.0)
        (Up, Vp), _ = solve(fields_for(m, ssa, H + h * d)[0])
        (Um, Vm), _ = solve(fields_for(m, ssa, H - h * d)[0])
        fd = (adj.misfit(Up, Vp, Uo, Vo) - adj.misfit(Um, Vm, Uo, Vo)) / (2 * h)
        an = float(dHi @ d)
        assert abs(fd - an) <= 1e-5 * abs(an), (fd, an)


def bed_fields_for(m, ssa, Hb):
    """Solve inputs for another bed (the geometry recomputed by the oracle)."""
    g = orc.update_geometry(m, ssa["Hi"], Hb, ssa["SL"])
    f = dict(ssa)
    for k in ("Hb_Ac", "dHs_dx_shelf", "dHs_dy_shelf", "dHs_dx_shelf_Ac", "dHs_dy_shelf_Ac"):
        f[k] = g[k]
    f["Hb"] = Hb
    return f, g


def test_coulomb_friction_gradient_matches_finite_differences_of_the_bed(coulomb):
    """dJ/dlog(tau_c) under the Coulomb law, checked through the reference's own friction input:
    the bed Hb sets tau_c (basal_yield_stress: the till friction angle and the pore-water
    fraction) and the surface slope of grounded ice. The chain dJ/dHb = dJ/dlog(tau_c) dlog(tau_c)/dHb
    + slope terms against central finite differences of the oracle's forward solve, on
    perturbations of vertices away from the floatation threshold (masks frozen)."""
    m, ssa, solve, U, V, out = coulomb
    H = np.asarray(ssa["Hi"], dtype=np.float64)
    Hb, SL = np.asarray(ssa["Hb"], dtype=np.float64), np.asarray(ssa["SL"], dtype=np.float64)
    x, y = m.base.V[:, 0], m.base.V[:, 1]
    bump = 20.0 * np.exp(-((x - 2e5) ** 2 + (y + 1e5) ** 2) / (2 * (1.5e5) ** 2))
    # observations from a thicker dome (a misfit well above the solver's tolerance)
    (Uo, Vo), _ = solve(fields_for(m, ssa, np.where(H > 0, H + bump, H))[0])
    lin = adj.Linearisation(m, ssa, U, V, tau_c=out["tau_c_AaAc"])
    gU, gV = U - Uo, V - Vo
    mx, my, dlt, dHi, sens = adj.adjoint_gradient(lin, gU, gV)
    dHb = adj.coulomb_bed_gradient(m, ssa, dlt, sens["hx"], sens["hy"])
    flot = (SL - Hb) * adj.RHO_SW / adj.RHO_I
    safe = (H > 50.0) & (np.abs(H - flot) > 50.0) & (np.abs(Hb) > 1.0)
    rng = np.random.default_rng(21)
    h = 1e-3   # the friction law's curvature in the bed (tan, the pore-water fraction, S(u)) wants a short step
    for _ in range(2):
        d = np.where(safe, rng.normal(size=H.size), 0.0)
        (Up, Vp), _ = solve(bed_fields_for(m, ssa, Hb + h * d)[0])
        (Um, Vm), _ = solve(bed_fields_for(m, ssa, Hb - h * d)[0])
        fd = (adj.misfit(Up, Vp, Uo, Vo) - adj.misfit(Um, Vm, Uo, Vo)) / (2 * h)
        an = float(dHb @ d)
        assert abs(fd - an) <= 1e-5 * abs(an), (fd, an)
