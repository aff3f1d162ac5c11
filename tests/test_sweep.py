"""Packing of sweep instances into waves of batched contexts (host logic, no GPU)."""
import importlib

import pytest

sweep = importlib.import_module("verkko-hem-repo_gb300.sweep")


def test_plan_waves_packs_consecutive_instances():
    sizes = [10, 20, 30, 5, 5, 40]
    assert sweep.plan_waves(sizes, 1.0, 1000.0) == [[0, 1, 2, 3, 4, 5]]
    assert sweep.plan_waves(sizes, 1.0, 40.0) == [[0, 1], [2, 3, 4], [5]]
    assert sweep.plan_waves(sizes, 2.0, 80.0) == [[0, 1], [2, 3, 4], [5]]
    waves = sweep.plan_waves(sizes, 1.0, 45.0)
    assert [i for w in waves for i in w] == list(range(len(sizes)))
    assert all(sum(sizes[i] for i in w) <= 45.0 for w in waves)


def test_plan_waves_rejects_oversized_instance():
    with pytest.raises(ValueError, match="instance 2"):
        sweep.plan_waves([10, 20, 50], 1.0, 40.0)
    assert sweep.plan_waves([], 1.0, 1.0) == []
