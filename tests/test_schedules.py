"""Host-side schedules of the mixed-precision path, checked on CPU through the library's own
code: the refinement's triangular-solve task lists (deadlock-free under in-order dispatch)
and the row groups of the host-buffer Cholesky (the copy/factorization overlap)."""
import pytest

import palial_gb300 as P


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("mt,nbl", [(1, 8), (2, 8), (5, 4), (16, 8), (64, 8), (33, 16)])
def test_solve_task_lists_are_deadlock_free(mt, nbl, kind):
    assert P.check_solve_tasks(mt, nbl, kind) == 0


@pytest.mark.parametrize("n,nb", [(32768, 512), (4096, 512), (1536, 512), (2048, 1024), (32768, 256), (65536, 512)])
def test_row_groups_cover_the_rows_and_join_in_time(n, nb):
    mt = n // nb
    groups = P.row_groups(n, nb)
    assert groups[0][0] == 0 and groups[0][1] >= min(2, mt) and groups[-1][1] == mt
    for (a0, a1, _, _), (b0, _, _, _) in zip(groups, groups[1:]):
        assert a1 == b0 and a1 > a0  # contiguous, non-empty
    dues = [g[2] for g in groups]
    assert dues == sorted(dues)
    for gs, ge, due, kg in groups[1:]:
        # a group joins the trailing updates no later than two steps before the front reaches it
        assert 0 <= kg <= max(0, gs - 2)
    assert len(groups) <= 64


def test_row_groups_reject_bad_sizes():
    with pytest.raises(P.PalialError):
        P.row_groups(1000, 512)


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("n,nb", [(32768, 512), (4096, 512), (1536, 512), (2048, 512), (16384, 1024),
                                  (32768, 256), (65536, 512), (8192, 256)])
def test_arrival_plan_is_consistent(n, nb, mode):
    """Each group's data is awaited before its first update, its skipped steps are applied in
    order exactly once, it joins by step gs - 2, and every rest update covers row k + 2."""
    assert P.check_arrival_plan(n, nb, mode) == 0
