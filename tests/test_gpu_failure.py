"""Failure detection without a GPU fault (run with -m gpu). Every device-side wait of the
solvers — team barriers, neighbour progress waits, the mixed sweeps' lagged decisions — is
bounded by a globaltimer limit. With the limit set to a few nanoseconds (UFE_WAIT_TIMEOUT_NS,
test-only) the waits run out: the CTA that gives up records UFE_TIMEOUT and sets the team's error
bit, which ends every other wait, and the kernel returns. The host reports UFE_TIMEOUT, and the
context stays usable: the next solve under the normal limit gives the same result as before."""
import numpy as np
import pytest

from conftest import oracle_aaac, oracle_inputs

from ufemism_gb300 import _native as nat
from ufemism_gb300 import api
from ufemism_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def device():
    api.init(0)


@pytest.mark.parametrize("precision", [nat.UFE_MIXED, nat.UFE_FP64])
def test_wait_timeout_reported_and_context_usable(precision, monkeypatch):
    m = oracle_aaac("4k")
    ssa, sia, g = oracle_inputs(m)
    p = api.default_params(precision=precision)
    dm = api.DeviceMesh(m)
    rc0, o0, s0 = dm.solve_ssa(ssa, p)
    monkeypatch.setenv("UFE_WAIT_TIMEOUT_NS", "5")
    rc1, o1, s1 = dm.solve_ssa(ssa, p, check=False)
    assert rc1 == nat.UFE_TIMEOUT
    assert "timed out" in nat.last_error()
    monkeypatch.delenv("UFE_WAIT_TIMEOUT_NS")
    rc2, o2, s2 = dm.solve_ssa(ssa, p)
    assert rc2 == rc0 and s2["sweeps"] == s0["sweeps"]
    for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac"):
        assert np.array_equal(o2[k], o0[k]), k
    dm.close()


def test_batched_wait_timeout_reported(monkeypatch):
    members = [wl.ensemble_member(n, 7100 + i) for i, n in enumerate((1500, 3000, 2200))]
    p = api.default_params(precision=nat.UFE_MIXED, sliding_law=nat.UFE_SLIDING_LINEAR)
    monkeypatch.setenv("UFE_WAIT_TIMEOUT_NS", "5")
    b = api.Batch([mesh for _, mesh, _ in members])
    for i, (_, _, f) in enumerate(members):
        b.upload(i, f, p)
    rc, stats, timing = b.run(p, check=False)
    b.close()
    assert rc == nat.UFE_TIMEOUT
    monkeypatch.delenv("UFE_WAIT_TIMEOUT_NS")
    base, mesh, f = members[0]
    dm = api.DeviceMesh(mesh)
    rc, out, st = dm.solve_ssa(f, p)
    assert rc >= 0 and np.all(np.isfinite(out["U_SSA"]))
    dm.close()
