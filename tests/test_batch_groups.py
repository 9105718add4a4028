"""Host logic of the batched sweep's concurrent groups (no GPU): the
lattices are split into groups of about the same number of cells, every
lattice in exactly one group, in ascending order within a group."""
import types

import pytest

from lbm_gb300.batch import Batch, sweep_apps


def _fake(cells):
    return types.SimpleNamespace(engines=[types.SimpleNamespace(N=c) for c in cells])


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_groups_partition_and_balance(n):
    apps = sweep_apps(seed=2024)
    cells = [a.nx * a.ny for a in apps]
    groups = Batch.groups(_fake(cells), n)
    flat = sorted(i for g in groups for i in g)
    assert flat == list(range(len(cells)))
    assert all(g == sorted(g) for g in groups)
    assert len(groups) == n
    sums = [sum(cells[i] for i in g) for g in groups]
    # greedy largest-first: no group exceeds another by more than the
    # largest lattice
    assert max(sums) - min(sums) <= max(cells)
    assert max(sums) / min(sums) < 1.02


def test_groups_more_than_lattices():
    groups = Batch.groups(_fake([100, 50]), 4)
    assert sorted(i for g in groups for i in g) == [0, 1]
    assert all(groups)
