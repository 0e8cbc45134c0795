"""Discretisation convergence of the neighbour functions on CPU: the oracle's averaged-gradient
first derivatives (get_neighbour_functions_vertex_gr, mesh_derivatives_module.f90:76-313) of
f = sin(kx) cos(ky) on seeded jittered meshes of about 2k, 8k and 32k vertices — the study the
reference's manual shows as figures (documentation/UFEMISM_documentation.tex:1912-1930). The RMS
error over the interior vertices falls by at least 1.7x per halving of the spacing (first order
on irregular meshes; measured 2.1x), from about 2 % at 2k vertices."""
import numpy as np

import oracle as orc
from ufemism_gb300.meshgen import sized_mesh


def _derivative_error(n):
    base = sized_mesh(n, 11)
    m = orc.build_aaac(base, colour=False)
    k = 2.0 * np.pi / 1500e3
    x, y = base.V[:, 0], base.V[:, 1]
    f = np.sin(k * x) * np.cos(k * y)
    fx = k * np.cos(k * x) * np.cos(k * y)
    fy = -k * np.sin(k * x) * np.sin(k * y)
    nC = np.asarray(base.nC)
    C = np.asarray(base.C) - 1
    Nx, Ny = np.asarray(m.Nx), np.asarray(m.Ny)
    rows = np.arange(base.nV)
    dx = Nx[rows, nC] * f           # the home coefficient sits at column nC + 1 (1-based)
    dy = Ny[rows, nC] * f
    for c in range(C.shape[1]):
        ok = c < nC
        dx[ok] += Nx[ok, c] * f[C[ok, c]]
        dy[ok] += Ny[ok, c] * f[C[ok, c]]
    inner = np.asarray(base.edge_index) == 0
    return float(np.sqrt(np.mean((dx - fx)[inner] ** 2 + (dy - fy)[inner] ** 2)) / k)


def test_first_derivatives_converge_with_refinement():
    e = [_derivative_error(n) for n in (2000, 8000, 32000)]
    assert e[0] < 0.025, e
    assert e[0] / e[1] > 1.7 and e[1] / e[2] > 1.7, e
