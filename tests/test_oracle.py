"""Known-answer tests that pin the CPU oracle (the reference ships no tests or golden vectors).

* the reference's own five-vertex dummy mesh (mesh_creation_module.f90:1896-2000): Ac
  numbering, Aci, edge indices and neighbour functions derived by hand;
* averaged-gradient neighbour functions reproduce linear fields exactly (Berends et al. 2021);
* check_solution invariant of the five-colouring;
* SIA against the analytic isothermal SIA velocity of the dome;
* the golden fixture committed under tests/golden (made by tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

from conftest import base_mesh, dummy_mesh, oracle_aaac, oracle_inputs, rel_l2

import oracle as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "tiny_dome.npz")


def test_dummy_mesh_ac_numbering():
    m = orc.build_aaac(dummy_mesh())
    assert m.nAc == 8 and m.nVAaAc == 13
    # visiting order vi = 1..5, ci = 1..nC(vi): (1,2) (1,5) (1,4) (2,3) (2,5) (3,4) (3,5) (4,5)
    pairs = [tuple(m.Aci[a, :2]) for a in range(8)]
    assert pairs == [(1, 2), (1, 5), (1, 4), (2, 3), (2, 5), (3, 4), (3, 5), (4, 5)]
    assert m.iAci[0, :3].tolist() == [1, 2, 3]
    assert m.iAci[1, :3].tolist() == [4, 5, 1]
    assert m.iAci[2, :3].tolist() == [6, 7, 4]
    assert m.iAci[3, :3].tolist() == [3, 8, 6]
    assert m.iAci[4, :4].tolist() == [2, 5, 7, 8]
    # edge Ac vertices: S, W, E, N sides; diagonals free
    assert m.edge_index_Ac.tolist() == [5, 0, 7, 3, 0, 1, 0, 0]
    # (1,5): triangle (4,1,5) has 1->5 counter-clockwise (vl = 4), (1,2,5) has 5->1 (vr = 2)
    assert m.Aci[1].tolist() == [1, 5, 4, 2]
    # boundary segment (1,2): single triangle (1,2,5), 4th entry 1
    assert m.Aci[0].tolist() == [1, 2, 5, 1]
    # combined mesh: Aa rows list their Ac ids + nV
    assert m.nCAaAc[:5].tolist() == [3, 3, 3, 3, 4]
    assert m.CAaAc[4, :4].tolist() == [2 + 5, 5 + 5, 7 + 5, 8 + 5]
    # edge Ac (1,2) on the south side: the pair is swapped so that x(vi) > x(vj), then it is
    # surrounded counter-clockwise by [2, Ac(5,2), Ac(5,1), 1]
    assert m.nCAaAc[5] == 4 and m.CAaAc[5, :4].tolist() == [2, 5 + 5, 2 + 5, 1]
    # free Ac (1,5): [vi, Ac(vr,vi), Ac(vr,vj), vj, Ac(vl,vj), Ac(vl,vi)] with vl = 4, vr = 2
    assert m.nCAaAc[6] == 6 and m.CAaAc[6, :6].tolist() == [1, 1 + 5, 5 + 5, 5, 8 + 5, 3 + 5]


def test_dummy_mesh_neighbour_functions():
    m = orc.build_aaac(dummy_mesh())
    # centre vertex (0,0), neighbours at the corners (Eqs. A1, A3, A7): home 0, x-weights
    # -1/4, 1/4, 1/4, -1/4 and y-weights -1/4, -1/4, 1/4, 1/4
    assert m.Nx[4, :5].tolist() == [-0.25, 0.25, 0.25, -0.25, 0.0]
    assert m.Ny[4, :5].tolist() == [-0.25, -0.25, 0.25, 0.25, 0.0]


def _nf_exact(m, ncheck=400):
    """Neighbour functions reproduce linear fields: sum N = 0, sum N x = 1, sum N y = 0."""
    V = np.asarray(m.VAaAc)
    rows = np.linspace(0, m.nVAaAc - 1, min(ncheck, m.nVAaAc)).astype(int)
    for ai in rows:
        n = m.nCAaAc[ai]
        nb = m.CAaAc[ai, :n] - 1
        nx = np.append(m.Nx_AaAc[ai, :n], m.Nx_AaAc[ai, n])
        ny = np.append(m.Ny_AaAc[ai, :n], m.Ny_AaAc[ai, n])
        xs = np.append(V[nb, 0], V[ai, 0])
        ys = np.append(V[nb, 1], V[ai, 1])
        scale = np.abs(nx).max() * 1500e3
        assert abs(nx.sum()) <= 1e-12 * scale
        assert abs(nx @ xs - 1.0) <= 1e-9 and abs(nx @ ys) <= 1e-9
        assert abs(ny @ ys - 1.0) <= 1e-9 and abs(ny @ xs) <= 1e-9


@pytest.mark.parametrize("name", ["tiny", "1k"])
def test_neighbour_functions_linear_exact(name):
    _nf_exact(oracle_aaac(name))


def test_neighbour_functions_second_order_interior():
    """Second-order functions of a free vertex on a regular hexagon give exact curvatures of
    a quadratic (the averaged-gradient scheme is exact for quadratics on symmetric stencils)."""
    ang = np.arange(6) * np.pi / 3
    vc = np.stack([np.cos(ang), np.sin(ang)], axis=1)
    Nx, Ny, Nxx, Nxy, Nyy = orc.neighbour_functions_vertex([0.0, 0.0], vc, False)
    xs = np.append(vc[:, 0], 0.0)
    ys = np.append(vc[:, 1], 0.0)
    for f, (exx, exy, eyy) in ((xs * xs, (2, 0, 0)), (xs * ys, (0, 1, 0)), (ys * ys, (0, 0, 2))):
        assert abs(Nxx @ f - exx) < 1e-12
        assert abs(Nxy @ f - exy) < 1e-12
        assert abs(Nyy @ f - eyy) < 1e-12


@pytest.mark.parametrize("name", ["tiny", "1k", "4k"])
def test_five_colouring_valid(name):
    m = oracle_aaac(name)
    assert m.colour_status == orc.OR_OK, "colouring reached an abort of the reference"
    assert m.colour_nV.sum() == m.nVAaAc
    for ai in range(m.nVAaAc):
        n = m.nCAaAc[ai]
        assert m.colour[ai] in (1, 2, 3, 4, 5)
        assert np.all(m.colour[m.CAaAc[ai, :n] - 1] != m.colour[ai])
    for c in range(5):
        lst = m.colour_vi[: m.colour_nV[c], c]
        assert np.all(np.diff(lst) > 0) and np.all(m.colour[lst - 1] == c + 1)


def test_sia_matches_analytic_dome():
    """SIA against u = -2A(rho g)^n/(n+2) H^(n+1) |grad h|^(n-1) grad h: the 15-level
    trapezoid quadrature of A zeta^3 differs from the exact integral by a fixed factor."""
    m = oracle_aaac("4k")
    ssa, sia, g = oracle_inputs(m)
    p = orc.default_params()
    out = orc.solve_sia(m, sia, p)
    A, rg = 1e-16, 910.0 * 9.81
    H = g["Hi_Ac"]
    sx, sy = g["dHs_dx_Ac"], g["dHs_dy_Ac"]
    smag2 = g["dHs_dp_Ac"] ** 2 + g["dHs_do_Ac"] ** 2
    u_exact = -2 * A * rg ** 3 / 5 * H ** 4 * smag2 * sx
    # discrete vertical factor: trapezoid double integral of zeta^3 on the zeta grid
    z = orc.ZETA_DEFAULT
    f = z ** 3
    integ = np.zeros_like(z)
    for k in range(len(z) - 2, -1, -1):
        integ[k] = integ[k + 1] - 0.5 * (f[k + 1] + f[k]) * (z[k + 1] - z[k])
    avg = np.sum(0.5 * (integ[1:] + integ[:-1]) * np.diff(z))
    factor = avg / (-0.2)  # the exact double integral of zeta^3 is -1/5
    sheet = sia["mask_sheet_Ac"] == 1
    ratio = out["Ux_SIA_Ac"][sheet & (np.abs(u_exact) > 1)] / u_exact[sheet & (np.abs(u_exact) > 1)]
    assert np.allclose(ratio, factor, rtol=1e-10)
    assert 0.95 < factor < 1.05


def test_neumann_edges_and_corners():
    m = oracle_aaac("tiny")
    rng = np.random.default_rng(3)
    d = rng.normal(size=m.nVAaAc)
    out = orc.neumann(m, d)
    nV = m.base.nV
    is_edge = np.concatenate([m.base.edge_index > 0, m.edge_index_Ac > 0])
    for ai in range(4, m.nVAaAc):
        if not is_edge[ai]:
            assert out[ai] == d[ai]
            continue
        nb = m.CAaAc[ai, : m.nCAaAc[ai]] - 1
        nb = nb[~is_edge[nb]]
        assert np.isclose(out[ai], d[nb].mean(), rtol=1e-14, atol=1e-15)
    for ai in range(4):
        nb = m.CAaAc[ai, : m.nCAaAc[ai]] - 1
        assert np.isclose(out[ai], out[nb].mean(), rtol=1e-14, atol=1e-15)


def test_ssa_converges_and_dome_is_symmetric():
    m = oracle_aaac("tiny")
    ssa, sia, g = oracle_inputs(m)
    rc, out, st = orc.solve_ssa(m, ssa, orc.default_params())
    assert rc == orc.OR_OK
    assert st["picard_iterations"] >= 2 and st["last_RN"] < 1e-3
    # flow is outward and radial on the grounded dome
    x, y = m.base.V[:, 0], m.base.V[:, 1]
    r = np.hypot(x, y)
    sel = (r > 150e3) & (r < 600e3) & (m.base.edge_index == 0)
    ur = (out["U_SSA"][sel] * x[sel] + out["V_SSA"][sel] * y[sel]) / r[sel]
    assert np.all(ur > 0)


def test_golden_fixture():
    """The oracle reproduces the committed golden fixture: mesh indexing and colouring bit
    for bit, floating point to 1e-12 (the fixture was made on another CPU architecture)."""
    if not os.path.exists(GOLDEN):
        pytest.skip("golden fixture not generated")
    gz = np.load(GOLDEN)
    m = oracle_aaac("tiny")
    for k in ("iAci", "Aci", "edge_index_Ac", "nCAaAc", "CAaAc", "colour", "colour_vi", "colour_nV"):
        assert np.array_equal(np.asarray(getattr(m, k)), gz[k]), k
    for k in ("Nx_AaAc", "Ny_AaAc", "Nxx_AaAc", "Nxy_AaAc", "Nyy_AaAc"):
        a, b = np.asarray(getattr(m, k)), gz[k]
        fin = np.isfinite(b)
        assert np.array_equal(np.isfinite(a), fin)
        assert np.allclose(a[fin], b[fin], rtol=1e-12, atol=0)
    ssa, sia, g = oracle_inputs(m)
    rc, out, st = orc.solve_ssa(m, ssa, orc.default_params())
    assert st["sweeps"] == gz["sweeps"].tolist()
    assert rel_l2(out["U_SSA"], gz["U_SSA"]) < 1e-12
    assert rel_l2(out["Uy_SSA_Ac"], gz["Uy_SSA_Ac"]) < 1e-12
    so = orc.solve_sia(m, sia, orc.default_params())
    assert rel_l2(so["Ux_SIA_Ac"], gz["Ux_SIA_Ac"]) < 1e-12


def test_derivatives_converge_under_refinement():
    """The discretisation study of the reference manual (averaged-gradient derivatives of
    f = sin x cos y, UFEMISM_documentation.tex:1912-1930), as numbers: the AaAc first
    derivatives of a smooth field converge as the seeded dome meshes refine."""
    errs = []
    for name in ("tiny", "1k", "4k"):
        m = oracle_aaac(name)
        xy = np.asarray(m.VAaAc)
        L = 300e3
        f = np.sin(xy[:, 0] / L) * np.cos(xy[:, 1] / L)
        fx = np.cos(xy[:, 0] / L) * np.cos(xy[:, 1] / L) / L
        fy = -np.sin(xy[:, 0] / L) * np.sin(xy[:, 1] / L) / L
        dx, dy = orc.ddx_ddy_aaac(m, f)
        edge = np.concatenate([m.base.edge_index > 0, m.edge_index_Ac > 0])
        e = np.sqrt(np.mean((dx - fx)[~edge] ** 2 + (dy - fy)[~edge] ** 2)) / np.sqrt(np.mean(fx ** 2 + fy ** 2))
        errs.append(e)
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 0.05
