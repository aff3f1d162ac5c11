"""Packing of sweep instances into waves of batched contexts, and the handoff of stalled
instances to contexts of their own (host logic, no GPU)."""
import dataclasses
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
            self.handoff = False

        def set_mg_handoff(self, on=True):
            self.handoff = bool(on)

        @property
        def handed_off(self):
            return np.zeros(len(self.params), bool)

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


@dataclasses.dataclass
class _Prm:
    k: int
    precision: int = 1
    mg_pre: int = 1
    mg_post: int = 1


class _HandoffGL(_FakeGL):
    """Instances in HARD stall in a batched context with handoff on: they stop after 2 Newton
    steps with a large residual and their state moved by 100.  Alone, those in HARDER stall
    again unless the context is FP64; everything else converges in 3 steps, adding 1000 to
    its state."""
    FP64 = 0
    MIXED = 1
    HARD = {1, 4}
    HARDER = {4}

    class FemGL(_FakeGL.FemGL):
        def _stalls(self, p):
            if len(self.params) > 1:
                return p.k in _HandoffGL.HARD
            return p.k in _HandoffGL.HARDER and p.precision != _HandoffGL.FP64

        def run(self, max_newton, linear_tol, converge_acc, allow_unconverged):
            st = np.array([self.handoff and self._stalls(p) for p in self.params])
            self._handed = st
            return {"newton_its": np.where(st, 2, 3).astype(np.int32), "gmres_its": np.where(st, 50, 20).astype(np.int32),
                    "residual": np.where(st, 1e-3, 1e-11), "converged": not st.any()}

        @property
        def handed_off(self):
            return self._handed.copy()

        def free_energy(self):
            return np.array([p.k for p in self.params], float)

        def event_stop(self):
            return 10.0 if len(self.params) == 1 else 1.0

        def solution(self):
            off, out = 0, self.x.copy()
            for m, st in zip(self.meshes, self._handed):
                out[off:off + 18 * m.nn] += 100.0 if st else 1000.0
                off += 18 * m.nn
            return out


def test_solve_sweep_hands_off_stalled_instances():
    """A wave's stalled instances leave it at the state they reached and are finished alone:
    first with two pre- and post-sweeps (handoff on), then in FP64; their counts add up, their
    device time is charged to their wave, the others are untouched."""
    sizes = [4, 6, 3, 5, 2]
    meshes = [_FakeMesh(n) for n in sizes]
    params = [_Prm(k) for k in range(len(sizes))]
    x0 = [np.full(18 * n, float(k)) for k, n in enumerate(sizes)]
    _FakeGL.created = []
    r = sweep.solve_sweep(_HandoffGL, meshes, params, x0, budget=1e9, keep_solutions=True)
    assert r["waves"] == [5]
    assert list(np.flatnonzero(r["handed_off"])) == [1, 4] and r["converged"].all()
    # instance 1: wave (2) + alone with 2/2 sweeps (3); instance 4: wave (2) + 2/2 sweeps
    # (stalls: 2) + FP64 (3)
    assert list(r["newton_its"]) == [3, 5, 3, 3, 7]
    assert list(r["gmres_its"]) == [20, 70, 20, 20, 120]
    assert r["handoff_ms"] == [30.0] and r["solve_ms"] == [31.0]
    finish = _FakeGL.created[3:]
    assert [(p.k, p.precision, p.mg_pre, p.mg_post) for (p,) in finish] == [(1, 1, 2, 2), (4, 1, 2, 2), (4, 0, 2, 2)]
    # the finish starts from the state the wave reached (+100), then converges (+1000)
    assert np.array_equal(r["solutions"][1], np.full(18 * 6, 1.0 + 100 + 1000))
    assert np.array_equal(r["solutions"][4], np.full(18 * 2, 4.0 + 100 + 100 + 1000))
    assert np.array_equal(r["solutions"][0], np.full(18 * 4, 1000.0))
    # without handoff nothing is handed off
    r2 = sweep.solve_sweep(_HandoffGL, meshes, params, x0, budget=1e9, handoff=False)
    assert not r2["handed_off"].any() and r2["handoff_ms"] == [0.0]
