"""GPU VJP of the converged SSA solve through the C-ABI (run with -m gpu), against the FP64
CPU adjoint reference evaluated at the GPU's converged velocities (which itself is pinned
against finite differences in test_adjoint_oracle.py), and against central finite
differences (h = 1e-4) of the GPU forward solve. Tolerances: adjoint state and gradients
1e-8 relative L2 against the reference; directional derivatives 1e-5 against finite
differences."""
import numpy as np
import pytest

from conftest import oracle_aaac, oracle_inputs, rel_l2

import oracle as orc
import ssa_adjoint as adj
from ufemism_gb300 import _native as nat
from ufemism_gb300 import api
from ufemism_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TIGHT = dict(SSA_RN_tol=1e-13, SSA_max_residual_UV=1e-11, SSA_max_outer_loops=300, SSA_max_inner_loops=1000000)
REF_TOL = 1e-8
FD_TOL = 1e-5


def setup_case(name, kind):
    api.init(0)
    m = oracle_aaac(name)
    ssa, sia, g = oracle_inputs(m, kind)
    logb = wl.log_beta_field(m, std=1.0, ell=100e3, seed=5)
    dm = api.DeviceMesh(m)
    p = api.default_params(precision=nat.UFE_FP64, **TIGHT)

    def solve(lb, fields=None):
        f = dict(fields or ssa)
        f["beta_sq_AaAc"] = np.exp(lb)
        rc, out, st = dm.solve_ssa(f, p)
        assert rc == 0 and st["last_RN"] < 1e-12, st
        return adj.aaac_velocity(out), f

    (Uo, Vo), _ = solve(logb + wl.log_beta_field(m, std=0.3, ell=100e3, seed=11))
    (U, V), f0 = solve(logb)          # the handle now holds the solve the VJP differentiates
    return m, ssa, logb, dm, p, solve, U, V, f0, Uo, Vo


def split(m, a):
    nV = m.base.nV
    return a[:nV], a[nV:]


@pytest.mark.parametrize("method", [nat.UFE_VJP_GMRES, nat.UFE_VJP_SOR])
@pytest.mark.parametrize("name,kind", [("1k", "dome"), ("1k", "marine")])
def test_vjp_matches_cpu_reference_and_finite_differences(name, kind, method):
    m, ssa, logb, dm, p, solve, U, V, f0, Uo, Vo = setup_case(name, kind)
    gU, gV = U - Uo, V - Vo
    dJ = dict(zip(("U_SSA", "Ux_SSA_Ac"), split(m, gU)))
    dJ.update(zip(("V_SSA", "Uy_SSA_Ac"), split(m, gV)))
    rc, out, st = dm.ssa_vjp(dJ, p, geom_mesh=m, method=method)
    assert rc == nat.UFE_OK, st
    # CPU reference at the GPU's converged state
    lin = adj.Linearisation(m, f0, U, V)
    G = adj.geometry_matrix(m, ssa["Hi"], ssa["Hb"], ssa["SL"])
    mx, my, dlb, dHi, sens = adj.adjoint_gradient(lin, gU, gV, G)
    assert rel_l2(out["lambda_U_AaAc"], mx) <= REF_TOL
    assert rel_l2(out["lambda_V_AaAc"], my) <= REF_TOL
    assert rel_l2(out["dJ_dlogbeta_sq_AaAc"], dlb) <= REF_TOL
    assert rel_l2(out["dJ_dhx_AaAc"], sens["hx"]) <= REF_TOL
    assert rel_l2(out["dJ_dHi_AaAc"], sens["Hi"]) <= REF_TOL
    assert rel_l2(out["dJ_dHi"], dHi) <= REF_TOL
    # finite differences of the GPU forward solve
    rng = np.random.default_rng(3)
    h = 1e-4
    for _ in range(2):
        d = rng.normal(size=m.nVAaAc)
        (Up, Vp), _ = solve(logb + h * d)
        (Um, Vm), _ = solve(logb - h * d)
        fd = (adj.misfit(Up, Vp, Uo, Vo) - adj.misfit(Um, Vm, Uo, Vo)) / (2 * h)
        an = float(out["dJ_dlogbeta_sq_AaAc"] @ d)
        assert abs(fd - an) <= FD_TOL * abs(an), (fd, an)
    Hi = ssa["Hi"]
    for _ in range(2):
        d = rng.normal(size=m.base.nV) * (Hi > 50.0)
        gp = orc.update_geometry(m, Hi + h * d, ssa["Hb"], ssa["SL"])
        gm = orc.update_geometry(m, Hi - h * d, ssa["Hb"], ssa["SL"])
        assert np.array_equal(gp["mask_ocean"], gm["mask_ocean"])
        assert np.array_equal(gp["mask_ocean_Ac"], gm["mask_ocean_Ac"])
        res = []
        for H, gg in ((Hi + h * d, gp), (Hi - h * d, gm)):
            f = dict(ssa)
            for k in ("Hi_Ac", "dHs_dx_shelf", "dHs_dy_shelf", "dHs_dx_shelf_Ac", "dHs_dy_shelf_Ac"):
                f[k] = gg[k]
            f["Hi"] = H
            (Uh, Vh), _ = solve(logb, f)
            res.append(adj.misfit(Uh, Vh, Uo, Vo))
        fd = (res[0] - res[1]) / (2 * h)
        an = float(out["dJ_dHi"] @ d)
        assert abs(fd - an) <= FD_TOL * abs(an), (fd, an)
    dm.close()


def geometry_fields(m, ssa, Hi=None, Hb=None):
    """Solve inputs for another thickness or bed, the geometry recomputed by the oracle."""
    Hi = ssa["Hi"] if Hi is None else Hi
    Hb = ssa["Hb"] if Hb is None else Hb
    g = orc.update_geometry(m, Hi, Hb, ssa["SL"])
    f = dict(ssa, Hi=Hi, Hb=Hb)
    for k in ("Hi_Ac", "Hb_Ac", "dHs_dx_shelf", "dHs_dy_shelf", "dHs_dx_shelf_Ac", "dHs_dy_shelf_Ac"):
        f[k] = g[k]
    return f, g


@pytest.mark.parametrize("name,kind", [("1k", "dome"), ("1k", "marine")])
def test_coulomb_vjp_matches_cpu_reference_and_finite_differences(name, kind):
    """The reference's Coulomb_regularised law: the transposed sweep carries each grounded
    row's S'(u) block. Against the CPU reference at the GPU's converged state: the adjoint
    state, dJ/dlog(tau_c), dJ/dphi_fric, the driving-stress sensitivity and dJ/dHi (<= 1e-8).
    Against central finite differences of the GPU forward solve (<= 1e-5): dJ/dHi, and on the
    marine bed (away from the friction law's clamps at Hb = 0) dJ/dHb through tau_c and the
    surface slope, which checks the friction gradient through the reference's own input."""
    api.init(0)
    m = oracle_aaac(name)
    ssa, sia, g = oracle_inputs(m, kind)
    dm = api.DeviceMesh(m)
    p = api.default_params(precision=nat.UFE_FP64, sliding_law=nat.UFE_SLIDING_COULOMB_REGULARISED, **TIGHT)

    def solve(f):
        rc, out, st = dm.solve_ssa(f, p)
        assert rc == 0 and st["last_RN"] < 1e-12, st
        return adj.aaac_velocity(out), out

    H, Hb, SL = (np.asarray(ssa[k], dtype=np.float64) for k in ("Hi", "Hb", "SL"))
    x, y = m.base.V[:, 0], m.base.V[:, 1]
    bump = 20.0 * np.exp(-((x - 2e5) ** 2 + (y + 1e5) ** 2) / (2 * (1.5e5) ** 2))
    (Uo, Vo), _ = solve(geometry_fields(m, ssa, Hi=np.where(H > 0, H + bump, H))[0])
    (U, V), out0 = solve(ssa)           # the handle now holds the solve the VJP differentiates
    gU, gV = U - Uo, V - Vo
    dJ = dict(zip(("U_SSA", "Ux_SSA_Ac"), split(m, gU)))
    dJ.update(zip(("V_SSA", "Uy_SSA_Ac"), split(m, gV)))
    rc, vo, st = dm.ssa_vjp(dJ, p, geom_mesh=m)
    assert rc == nat.UFE_OK, st
    lin = adj.Linearisation(m, ssa, U, V, tau_c=out0["tau_c_AaAc"])
    assert np.any(lin.fr > 0)
    G = adj.geometry_matrix(m, H, Hb, SL)
    mx, my, dlt, dHi, sens = adj.adjoint_gradient(lin, gU, gV, G)
    assert rel_l2(vo["lambda_U_AaAc"], mx) <= REF_TOL
    assert rel_l2(vo["lambda_V_AaAc"], my) <= REF_TOL
    assert rel_l2(vo["dJ_dlogbeta_sq_AaAc"], dlt) <= REF_TOL
    assert rel_l2(vo["dJ_dhx_AaAc"], sens["hx"]) <= REF_TOL
    assert rel_l2(vo["dJ_dHi"], dHi) <= REF_TOL
    assert np.all(vo["dJ_dHi_AaAc"] == 0.0)     # the friction term does not depend on Hi
    r = np.pi / 180.0
    phi = out0["phi_fric_AaAc"]
    assert rel_l2(vo["dJ_dphi_fric_AaAc"], dlt * r / (np.sin(r * phi) * np.cos(r * phi))) <= REF_TOL
    rng = np.random.default_rng(17)
    h = 1e-3
    flot = (SL - Hb) * adj.RHO_SW / adj.RHO_I
    safe = (H > 50.0) & (np.abs(H - flot) > 50.0)
    J = lambda UV: adj.misfit(UV[0], UV[1], Uo, Vo)
    for _ in range(2):
        d = np.where(safe, rng.normal(size=H.size), 0.0)
        fp = solve(geometry_fields(m, ssa, Hi=H + h * d)[0])[0]
        fm = solve(geometry_fields(m, ssa, Hi=H - h * d)[0])[0]
        fd = (J(fp) - J(fm)) / (2 * h)
        an = float(vo["dJ_dHi"] @ d)
        assert abs(fd - an) <= FD_TOL * abs(an), (fd, an)
    if kind == "marine":
        dHb = adj.coulomb_bed_gradient(m, ssa, vo["dJ_dlogbeta_sq_AaAc"], vo["dJ_dhx_AaAc"], vo["dJ_dhy_AaAc"])
        for _ in range(2):
            d = np.where(safe & (np.abs(Hb) > 1.0), rng.normal(size=H.size), 0.0)
            fp = solve(geometry_fields(m, ssa, Hb=Hb + h * d)[0])[0]
            fm = solve(geometry_fields(m, ssa, Hb=Hb - h * d)[0])[0]
            fd = (J(fp) - J(fm)) / (2 * h)
            an = float(dHb @ d)
            assert abs(fd - an) <= FD_TOL * abs(an), (fd, an)
    dm.close()


def test_vjp_rejects_missing_solve_and_a_changed_law():
    api.init(0)
    m = oracle_aaac("tiny")
    dm = api.DeviceMesh(m)
    dJ = {k: np.zeros(n) for k, n in (("U_SSA", m.base.nV), ("V_SSA", m.base.nV), ("Ux_SSA_Ac", m.nAc),
                                      ("Uy_SSA_Ac", m.nAc))}
    rc, out, st = dm.ssa_vjp(dJ, api.default_params(), check=False)
    assert rc == nat.UFE_BAD_ARG
    ssa, sia, g = oracle_inputs(m, "dome")
    p = api.default_params(sliding_law=nat.UFE_SLIDING_COULOMB_REGULARISED)
    dm.solve_ssa(ssa, p)
    rc, out, st = dm.ssa_vjp(dJ, api.default_params(sliding_law=nat.UFE_SLIDING_LINEAR), check=False)
    assert rc == nat.UFE_BAD_ARG and "sliding law differs" in nat.last_error()
    dm.close()


def test_vjp_reports_divergence_and_recovers():
    """A relaxation factor far above the forward's makes the transposed SOR diverge on the
    marine case; the VJP reports UFE_DIVERGED (no GPU fault: the iteration stops on a
    non-finite reduction) and the handle stays usable."""
    m, ssa, logb, dm, p, solve, U, V, f0, Uo, Vo = setup_case("1k", "marine")
    gU, gV = U - Uo, V - Vo
    dJ = dict(zip(("U_SSA", "Ux_SSA_Ac"), split(m, gU)))
    dJ.update(zip(("V_SSA", "Uy_SSA_Ac"), split(m, gV)))
    rc, out, st = dm.ssa_vjp(dJ, p, omega=1.99, max_sweeps=200000, check=False, method=nat.UFE_VJP_SOR)
    assert rc in (nat.UFE_DIVERGED, nat.UFE_OK, nat.UFE_NOT_CONVERGED)
    if rc == nat.UFE_OK:   # converged after all: the gradient must then be right
        lin = adj.Linearisation(m, f0, U, V)
        mx, my, dlb, dHi, sens = adj.adjoint_gradient(lin, gU, gV)
        assert rel_l2(out["dJ_dlogbeta_sq_AaAc"], dlb) <= 1e-6
    rc2, out2, st2 = dm.ssa_vjp(dJ, p)
    assert rc2 == nat.UFE_OK
    dm.close()


def test_vjp_at_100k_matches_cpu_adjoint_and_tangent_linear():
    """The benchmark's adjoint size (100k-vertex marine setup, log-normal friction field): the
    GPU VJP against the CPU reference linearised at the GPU's own state, through one sparse LU
    of the Jacobian (about 0.8M unknowns) used both ways: the adjoint state and the gradients
    (transposed solve, <= 1e-8), and tangent-linear directional derivatives of J on random
    directions of log(beta^2) and of Hi against the VJP's gradients (<= 1e-8). Both sides
    linearise at the same velocities, so the forward solve runs at the default tolerances."""
    import scipy.sparse.linalg as spla
    api.init(0)
    m = oracle_aaac("100k")
    ssa, sia, g = oracle_inputs(m, "marine")
    lb = wl.log_beta_field(m, std=1.0, ell=100e3, seed=5)
    dm = api.DeviceMesh(m)
    p = api.default_params(precision=nat.UFE_MIXED)
    f_obs = dict(ssa, beta_sq_AaAc=np.exp(lb + wl.log_beta_field(m, std=0.3, ell=100e3, seed=11, mean=0.0)))
    rc, oo, _ = dm.solve_ssa(f_obs, p, check=False)
    f0 = dict(ssa, beta_sq_AaAc=np.exp(lb))
    rc, out, st = dm.solve_ssa(f0, p, check=False)
    U, V = adj.aaac_velocity(out)
    Uo, Vo = adj.aaac_velocity(oo)
    gU, gV = U - Uo, V - Vo
    dJ = dict(zip(("U_SSA", "Ux_SSA_Ac"), split(m, gU)))
    dJ.update(zip(("V_SSA", "Uy_SSA_Ac"), split(m, gV)))
    rcv, vo, vs = dm.ssa_vjp(dJ, p, geom_mesh=m)
    assert rcv == nat.UFE_OK, vs
    lin = adj.Linearisation(m, f0, U, V)
    K = lin.jacobian().tocsc()
    lu = spla.splu(K)
    nA = m.nVAaAc
    mu = lu.solve(np.concatenate([gU, gV]), trans="T")
    mx, my = mu[:nA], mu[nA:]
    assert rel_l2(vo["lambda_U_AaAc"], mx) <= REF_TOL
    assert rel_l2(vo["lambda_V_AaAc"], my) <= REF_TOL
    bx, by = lin.dF_dlogbeta()
    assert rel_l2(vo["dJ_dlogbeta_sq_AaAc"], -(mx * bx + my * by)) <= REF_TOL
    G = adj.geometry_matrix(m, ssa["Hi"], ssa["Hb"], ssa["SL"])
    Gx, Gy, GH = G
    dhx, dHx, dHy = lin.dF_dfields()
    rng = np.random.default_rng(29)
    for _ in range(4):
        d = rng.normal(size=nA)
        du = lu.solve(np.concatenate([-bx * d, -by * d]))
        tlm = float(gU @ du[:nA] + gV @ du[nA:])
        an = float(vo["dJ_dlogbeta_sq_AaAc"] @ d)
        assert abs(tlm - an) <= REF_TOL * abs(an), (tlm, an)
    for _ in range(2):
        d = rng.normal(size=m.base.nV) * (np.asarray(ssa["Hi"]) > 50.0)
        rhs = np.concatenate([-(dhx * (Gx @ d) + dHx * (GH @ d)), -(dhx * (Gy @ d) + dHy * (GH @ d))])
        du = lu.solve(rhs)
        tlm = float(gU @ du[:nA] + gV @ du[nA:])
        an = float(vo["dJ_dHi"] @ d)
        assert abs(tlm - an) <= REF_TOL * abs(an), (tlm, an)
    dm.close()
