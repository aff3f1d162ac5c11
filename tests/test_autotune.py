"""Autotuner: the coordinate descent and the problem signature on CPU (a fake timer), and
on the GPU a tuning run on a small cube whose result is cached and converges."""
import json

import pytest

from _lib import ROOT, product  # noqa: F401

import importlib
import sys

sys.path.insert(0, ROOT)
at = importlib.import_module("verkko-hem-repo_gb300.autotune")


def _fake(costs, fails=()):
    """measure(cfg) = base + per-field costs; configs listed in `fails` do not converge."""
    calls = []

    def measure(cfg):
        calls.append(dict(cfg))
        key = (cfg["precond"], cfg["gmres_restart"], cfg["mg_pre"], cfg["mg_post"], cfg["mf_cells"])
        if key in fails:
            return None
        return 100.0 + costs["precond"][cfg["precond"]] + costs["restart"][cfg["gmres_restart"]] + \
            costs["sweeps"][(cfg["mg_pre"], cfg["mg_post"])] + costs["cells"][cfg["mf_cells"]] + \
            costs.get("reuse", {}).get(cfg["prec_reuse"], 0.0)

    return measure, calls


COSTS = {"precond": {"mg": 0.0, "bj": 50.0}, "restart": {30: 5.0, 50: 0.0, 64: -8.0},
         "sweeps": {(1, 1): 0.0, (1, 0): 1.0, (2, 1): -3.0, (2, 2): 4.0}, "cells": {4: 6.0, 8: 0.0, 16: -10.0},
         "reuse": {0.0: 0.0, 1e-2: -2.0, 1e-1: -4.0, 1.0: 3.0}}


def test_search_finds_the_best_coordinates():
    measure, calls = _fake(COSTS)
    out = at.search(measure, margin=0.0)
    assert out["config"] == {"precond": "mg", "gmres_restart": 64, "mg_pre": 2, "mg_post": 1, "mf_cells": 16,
                             "prec_reuse": 1e-1}
    assert out["ms"] == pytest.approx(100.0 - 8.0 - 3.0 - 10.0 - 4.0)
    # one start plus the other values of each coordinate: 1 + 1 + 2 + 3 + 2 + 3
    assert len(calls) == 12 and len(out["trials"]) == 12


def test_search_margin_and_failures():
    # a 2% margin keeps the default when the gain is smaller
    small = {"precond": {"mg": 0.0, "bj": 50.0}, "restart": {30: 5.0, 50: 0.0, 64: -1.0},
             "sweeps": {(1, 1): 0.0, (1, 0): 0.5, (2, 1): 0.5, (2, 2): 0.5}, "cells": {4: 0.0, 8: 0.0, 16: 0.0}}
    measure, _ = _fake(small)
    assert at.search(measure, margin=0.02)["config"] == at.DEFAULT
    # a candidate that does not converge is skipped even when it would be fastest
    measure, _ = _fake(COSTS, fails={("mg", 64, 1, 1, 8)})
    out = at.search(measure, margin=0.0)
    assert out["config"]["gmres_restart"] == 50
    # without multigrid only block-Jacobi configurations are tried, and no sweeps
    measure, calls = _fake(COSTS)
    out = at.search(measure, margin=0.0, multigrid=False)
    assert all(c["precond"] == "bj" for c in calls) and out["config"]["precond"] == "bj"
    assert {(c["mg_pre"], c["mg_post"]) for c in calls} == {(1, 1)}
    assert {c["prec_reuse"] for c in calls} == {0.0}
    # a start that does not converge is an error
    with pytest.raises(RuntimeError):
        at.search(lambda cfg: None)


def test_signature():
    class M:
        def __init__(self, nn, nc, nh=0):
            self.nn, self.nc, self.n_hanging = nn, nc, nh

    a = at.signature([M(125, 64)], 1)
    assert a == at.signature([M(125, 64)], 1)
    assert a != at.signature([M(125, 64)], 0)
    assert a != at.signature([M(125, 64, 3)], 1)
    assert a != at.signature([M(125, 64), M(27, 8)], 1)


@pytest.mark.gpu
def test_tune_small_cube(tmp_path):
    gl = product()
    m = gl.cube_mesh(5.0, 8)
    prm = gl.Params.from_matep(20.0, 0.6, precision=gl.MIXED)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=2)
    cache = str(tmp_path / "tune.json")
    out = at.tune(gl, [m], [prm], x0, cache=cache)
    assert not out["cached"] and out["ms"] > 0 and len(out["trials"]) >= 6
    again = at.tune(gl, [m], [prm], x0, cache=cache)
    assert again["cached"] and again["config"] == out["config"]
    assert json.load(open(cache))[out["signature"]]["config"] == out["config"]
    with gl.FemGL(m, at.params_with(gl, prm, out["config"])) as f:
        f.set_solution(x0)
        res = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
    assert res["converged"]
