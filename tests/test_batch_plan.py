"""The ensemble planner (ufe_batch_plan) on the host: member team sizes, class teams and
the CTA budget. No GPU needed."""
import numpy as np
import pytest

from ufemism_gb300 import _native as nat
from ufemism_gb300 import api
from ufemism_gb300 import workloads as wl


def rows_of(n_vertices):
    return 4 * np.asarray(n_vertices, dtype=np.int64)   # nA = nV + nAc, nAc about 3 nV


def test_uniform_teams():
    rows = rows_of([2000, 5000, 50000])
    t, classes, grid = api.batch_plan(rows, 152, team_ctas=16)
    assert list(t) == [16, 16, 16]
    assert classes == [(16, 3)] and grid == 48


def test_packing_gives_power_of_two_teams_and_fits_budget():
    rows = rows_of(wl.ensemble_sizes(256))
    for R in (2048, 4096, 8192, 16384):
        for resident in (152, 304, 608):
            t, classes, grid = api.batch_plan(rows, resident, rows_per_cta=R)
            assert grid <= resident
            assert all(x & (x - 1) == 0 for x in t)
            # every member fits the per-CTA slice table and has at least 32 rows per patch
            assert np.all(rows / t <= 1024 * 32 * 3 // 4)
            assert np.all(rows // t >= 32)
            sizes = sorted(set(t.tolist()), reverse=True)
            assert [c[0] for c in classes] == sizes
            for size, teams in classes:
                assert 1 <= teams <= int(np.sum(t == size))
            assert grid == sum(s * k for s, k in classes)


def test_smaller_packing_means_larger_teams():
    rows = rows_of(wl.ensemble_sizes(64))
    t1, _, _ = api.batch_plan(rows, 608, rows_per_cta=16384)
    t2, _, _ = api.batch_plan(rows, 608, rows_per_cta=2048)
    assert np.all(t2 >= t1) and np.any(t2 > t1)


def test_plan_rejects_impossible_requests():
    with pytest.raises(nat.UfeError):
        api.batch_plan(rows_of([2000]), 152, team_ctas=400)        # more patches than rows allow
    with pytest.raises(nat.UfeError):
        api.batch_plan(rows_of([60000]), 152, team_ctas=1)         # one patch cannot hold 240k rows
    with pytest.raises(nat.UfeError):
        api.batch_plan(rows_of([2000]), 152, block=300)
