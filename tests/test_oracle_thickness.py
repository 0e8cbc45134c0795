"""The oracle's calculate_ice_thickness_change on CPU: volume conservation of the fluxes
(antisymmetric, so the summed volume change is the surface and basal balance), no negative
thickness after the outflux rescale, and the zero-time-step and domain-edge rules."""
import numpy as np

from conftest import oracle_aaac, oracle_inputs

import oracle as orc
from ufemism_gb300 import workloads as wl


def _case():
    m = oracle_aaac("1k")
    ssa, sia, g = oracle_inputs(m, "marine")
    A, Cw = wl.areas_and_widths(m.base)
    rng = np.random.default_rng(5)
    return (m, ssa, A, Cw, rng.normal(size=m.nAc) * 50, rng.normal(size=m.nAc) * 400,
            rng.normal(size=m.base.nV) * 0.5, -np.abs(rng.normal(size=m.base.nV)) * 20 * (ssa["Hi"] > 0))


def test_fluxes_are_antisymmetric_and_conserve_volume():
    m, ssa, A, Cw, us, uq, smb, bmb = _case()
    Hn, Hp, dh, dv = orc.thickness_change(m, A, Cw, us, uq, np.zeros_like(smb), np.zeros_like(bmb), 1.0,
                                          ssa["Hi"], zero_edges=False)
    # with no surface or basal balance, the volume change is the sum of fluxes: zero
    assert abs(np.sum(A * dh)) <= 1e-9 * np.sum(np.abs(dv))
    C = np.asarray(m.base.C) - 1
    for v in range(0, m.base.nV, 37):
        for c in range(m.base.nC[v]):
            w = C[v, c]
            cw = list(C[w, :m.base.nC[w]]).index(v)
            assert dv[v, c] == -dv[w, cw]


def test_rescale_prevents_negative_thickness_and_rules_apply():
    m, ssa, A, Cw, us, uq, smb, bmb = _case()
    Hn, Hp, dh, dv = orc.thickness_change(m, A, Cw, us, uq, smb, bmb, 500.0, ssa["Hi"])
    assert np.all(Hn >= -1e-9 * ssa["Hi"].max())
    assert np.all(Hn[m.base.edge_index > 0] == 0.0)
    assert np.array_equal(Hp, ssa["Hi"])
    H0, _, dh0, _ = orc.thickness_change(m, A, Cw, us, uq, smb, bmb, 0.0, ssa["Hi"], zero_edges=False)
    assert np.all(dh0 == 0.0) and np.array_equal(H0, ssa["Hi"])
