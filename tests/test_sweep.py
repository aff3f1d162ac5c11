"""Packing of sweep instances into waves of batched contexts (host logic, no GPU)."""
import importlib

import numpy as np
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


class _FakeMesh:
    def __init__(self, nn):
        self.nn = nn


class _FakeGL:
    """Stands in for the binding: a context's 'solution' is its start plus the instance id,
    its free energy the instance id, so the bookkeeping of every wave can be checked."""

    created = []

    @staticmethod
    def mem_info():
        return 10**9, 2 * 10**9

    class FemGL:
        def __init__(self, meshes, params):
            self.meshes = meshes if isinstance(meshes, list) else [meshes]
            self.params = params if isinstance(params, list) else [params]
            _FakeGL.created.append([p for p in self.params])
            self.device_bytes = 100 * sum(m.nn for m in self.meshes)
            self.mg_fallbacks = 0

        def __enter__(self):
            return self

        def __exit__(self, *a):
            self.close()

        def set_solution(self, x):
            self.x = np.array(x)

        def sync(self):
            pass

        def event_start(self):
            pass

        def event_stop(self):
            return 1.0

        def run(self, max_newton, linear_tol, converge_acc, allow_unconverged):
            k = len(self.params)
            return {"newton_its": np.array(self.params, np.int32), "gmres_its": np.full(k, 7, np.int32),
                    "residual": np.full(k, 1e-11), "converged": True}

        def free_energy(self):
            return np.array(self.params, float)

        def solution(self):
            off, out = 0, self.x.copy()
            for m, p in zip(self.meshes, self.params):
                out[off:off + 18 * m.nn] += p
                off += 18 * m.nn
            return out

        def close(self):
            pass


def test_solve_sweep_bookkeeping():
    sizes = [5, 9, 3, 7, 2, 8]
    meshes = [_FakeMesh(n) for n in sizes]
    params = list(range(len(sizes)))
    x0 = [np.full(18 * n, 0.5 * k) for k, n in enumerate(sizes)]
    _FakeGL.created = []
    r = sweep.solve_sweep(_FakeGL, meshes, params, x0, budget=100 * 1.1 * 12, keep_solutions=True)
    # the probes are the largest and the smallest instance; each wave holds at most 12
    # nodes (budget / margin)
    assert _FakeGL.created[0] == [1] and _FakeGL.created[1] == [4]
    waves = _FakeGL.created[2:]
    assert [i for w in waves for i in w] == params and r["waves"] == [len(w) for w in waves]
    assert all(sum(sizes[i] for i in w) <= 12 for w in waves)
    assert np.array_equal(r["newton_its"], params) and np.array_equal(r["free_energy"], params)
    for k, s in enumerate(r["solutions"]):
        assert np.array_equal(s, np.full(18 * sizes[k], 0.5 * k + k))
    assert r["converged"].all() and r["bytes_per_node"] == 100.0 and r["bytes_per_instance"] == 0.0
    assert [int(r["wave"][i]) for i in params] == [j for j, w in enumerate(waves) for _ in w]
    with pytest.raises(ValueError):
        sweep.solve_sweep(_FakeGL, meshes, params, x0[:-1])


def test_footprint_fits_a_constant_per_instance():
    """Small instances carry fixed costs (coarse levels, Krylov bookkeeping): the fit
    through the largest and the smallest probe recovers constant and slope, and the waves
    charge the constant to every instance."""

    class GL(_FakeGL):
        class FemGL(_FakeGL.FemGL):
            def __init__(self, meshes, params):
                super().__init__(meshes, params)
                self.device_bytes = 5000 * len(self.meshes) + 100 * sum(m.nn for m in self.meshes)

    meshes = [_FakeMesh(n) for n in (40, 2, 10, 25)]
    slope, const = sweep.footprint(GL, meshes, [0, 1, 2, 3])
    assert slope == pytest.approx(100.0) and const == pytest.approx(5000.0)
    # budget 16000: with the constant, at most two instances of <= 25 nodes share a wave
    waves = sweep.plan_waves([25, 2, 10, 25], slope, 16000.0, const)
    assert waves == [[0, 1], [2, 3]]
