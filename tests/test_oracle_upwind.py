"""The oracle's upwind derivatives (get_upwind_derivative_vertex_3D) on CPU: the triangle
functions and both branches (upwind triangle, no wind) reproduce linear fields, mesh%R is the
nearest-neighbour distance, the chosen triangle contains the upwind point, and an upwind point
is missed only on the domain edge (where the thermodynamics never asks)."""
import numpy as np
import pytest

from conftest import oracle_aaac

import oracle as orc


@pytest.fixture(scope="module")
def mesh():
    m = oracle_aaac("1k")
    NxT, NyT = orc.triangle_functions(m.base)
    R = orc.vertex_resolution(m.base)
    return m, NxT, NyT, R


def test_triangle_functions_and_resolution(mesh):
    m, NxT, NyT, R = mesh
    V = np.asarray(m.base.V)
    T = np.asarray(m.base.Tri) - 1
    f = 3.0 + 2e-5 * V[:, 0] - 7e-6 * V[:, 1]
    assert np.allclose((NxT * f[T]).sum(axis=1), 2e-5, rtol=1e-8, atol=0)
    assert np.allclose((NyT * f[T]).sum(axis=1), -7e-6, rtol=1e-8, atol=0)
    C = np.asarray(m.base.C) - 1
    nC = np.asarray(m.base.nC)
    for v in range(0, m.base.nV, 13):
        dv = V[C[v, :nC[v]]] - V[v]
        d = np.sqrt(dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1])
        assert R[v] == d.min()


def _winds(nV, nZ, rng):
    U = rng.normal(size=(nV, nZ)) * 100.0
    V = rng.normal(size=(nV, nZ)) * 100.0
    U[:, 0] = 0.0
    V[:, 0] = 0.0             # a layer without wind: the neighbour-function branch
    return np.asfortranarray(U), np.asfortranarray(V)


def test_linear_field_and_edge_only_misses(mesh):
    m, NxT, NyT, R = mesh
    nV, nZ = m.base.nV, 6
    Vx = np.asarray(m.base.V)
    U, V = _winds(nV, nZ, np.random.default_rng(3))
    d = np.asfortranarray(np.stack([1.0 + (k + 1) * 1e-5 * Vx[:, 0] - 3e-6 * Vx[:, 1] for k in range(nZ)], axis=1))
    ddx, ddy, missing = orc.upwind_derivatives_3d(m, R, NxT, NyT, U, V, d)
    edge = np.asarray(m.base.edge_index) > 0
    found = np.ones((nV, nZ), dtype=bool)
    # recompute which pairs had no triangle: their derivatives are exactly 0
    found[(ddx == 0.0) & (ddy == 0.0)] = False
    assert missing == int((~found).sum())
    assert found[~edge].all(), "an interior vertex without an upwind triangle"
    for k in range(nZ):
        ok = found[:, k]
        assert np.allclose(ddx[ok, k], (k + 1) * 1e-5, rtol=1e-7, atol=0), k
        assert np.allclose(ddy[ok, k], -3e-6, rtol=1e-7, atol=0), k


def test_chosen_triangle_contains_the_upwind_point(mesh):
    m, NxT, NyT, R = mesh
    nV = m.base.nV
    Vx = np.asarray(m.base.V)
    T = np.asarray(m.base.Tri) - 1
    iTri = np.asarray(m.base.iTri) - 1
    niTri = np.asarray(m.base.niTri)
    rng = np.random.default_rng(8)
    U, V = _winds(nV, 2, rng)
    interior = np.flatnonzero(np.asarray(m.base.edge_index) == 0)[::7]
    for vi in interior:
        u, v = U[vi, 1], V[vi, 1]
        p = Vx[vi] - np.array([u, v]) * R[vi] / (4.0 * np.sqrt(u * u + v * v))
        tri = [t for t in iTri[vi, :niTri[vi]]]
        inside = []
        for t in tri:
            a, b, c = Vx[T[t]]
            M = np.array([b - a, c - a]).T
            l1, l2 = np.linalg.solve(M, p - a)
            inside.append(min(l1, l2, 1 - l1 - l2) > -1e-9)
        assert any(inside)
        first = tri[int(np.argmax(inside))]
        # the derivative of the indicator of the chosen triangle's first corner is its NxTri entry
        d = np.zeros((nV, 2), order="F")
        d[T[first, 0], :] = 1.0
        Ux = np.zeros((nV, 2), order="F")
        Vy = np.zeros((nV, 2), order="F")
        Ux[vi, 1], Vy[vi, 1] = u, v
        ddx, ddy, _ = orc.upwind_derivatives_3d(m, R, NxT, NyT, Ux, Vy, d)
        assert ddx[vi, 1] == NxT[first, 0] and ddy[vi, 1] == NyT[first, 0]
