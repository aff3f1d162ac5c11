"""Autotuner for the solver's launch shapes and Krylov parameters.

The reference has no counterpart (its solver parameters come from the configuration file,
confreader/src/declare.cc:155-290).  For a given set of instance meshes and precision this
picks the configuration that solves fastest:

* the preconditioner: geometric multigrid where it applies (tensor box grids), or
  block-Jacobi;
* the GMRES restart length;
* the multigrid smoothing sweeps before / after the coarse correction;
* the cell batch of the matrix-free FP32 operator (cells per CTA: 4, 8 or 16);
* how small a Newton step must be for the next step to keep the multigrid preconditioner.

Each candidate is timed on one complete Newton solve of the instances from the given start
(CUDA events around ``run``, after a warm-up solve that also builds the CUDA graphs).
Candidates that do not converge are discarded.  A coordinate descent from the defaults
keeps the number of trials small, and a candidate replaces the current choice only when it
is more than ``margin`` faster.  Results are cached per problem signature in a JSON file.
"""
from __future__ import annotations

import hashlib
import json
import os
from typing import Callable, Optional, Sequence

DEFAULT = {"precond": "mg", "gmres_restart": 50, "mg_pre": 1, "mg_post": 1, "mf_cells": 8, "prec_reuse": 0.0}
SEARCH = (
    ("precond", ("mg", "bj")),
    ("gmres_restart", (30, 50, 64)),
    ("mg_sweeps", ((1, 1), (1, 0), (2, 1), (2, 2))),
    ("mf_cells", (4, 8, 16)),
    ("prec_reuse", (0.0, 1e-2, 1e-1, 1.0)),
)


def signature(meshes: Sequence, precision: int, extra: str = "") -> str:
    """Key of a problem: instance sizes (nodes, cells, hanging nodes), precision, extra."""
    sizes = [(int(m.nn), int(m.nc), int(m.n_hanging)) for m in meshes]
    blob = json.dumps({"sizes": sizes, "precision": int(precision), "extra": extra}, sort_keys=True)
    return hashlib.sha1(blob.encode()).hexdigest()[:16]


def _with(cfg: dict, key: str, value) -> dict:
    out = dict(cfg)
    if key == "mg_sweeps":
        out["mg_pre"], out["mg_post"] = value
    else:
        out[key] = value
    return out


def _value(cfg: dict, key: str):
    return (cfg["mg_pre"], cfg["mg_post"]) if key == "mg_sweeps" else cfg[key]


def search(measure: Callable[[dict], Optional[float]], start: Optional[dict] = None, margin: float = 0.02,
           multigrid: bool = True) -> dict:
    """Coordinate descent over SEARCH.  measure(cfg) returns milliseconds, or None when the
    candidate did not converge.  Returns {"config", "ms", "trials"}."""
    cfg = dict(DEFAULT if start is None else start)
    if not multigrid:
        cfg["precond"] = "bj"
    trials = []
    best = measure(cfg)
    trials.append({"config": dict(cfg), "ms": best})
    if best is None:
        raise RuntimeError("autotune: the starting configuration does not converge")
    for key, values in SEARCH:
        if key in ("mg_sweeps", "prec_reuse") and cfg["precond"] != "mg":
            continue
        if key == "precond" and not multigrid:
            continue
        for v in values:
            if v == _value(cfg, key):
                continue
            cand = _with(cfg, key, v)
            ms = measure(cand)
            trials.append({"config": dict(cand), "ms": ms})
            if ms is not None and ms < best * (1.0 - margin):
                cfg, best = cand, ms
    return {"config": cfg, "ms": best, "trials": trials}


def params_with(gl, params, cfg: dict):
    """A copy of Params with the tuned fields set."""
    import dataclasses

    pc = gl.PC_MULTIGRID if cfg["precond"] == "mg" else gl.PC_BLOCK_JACOBI
    return dataclasses.replace(params, precond=pc, gmres_restart=int(cfg["gmres_restart"]), mg_pre=int(cfg["mg_pre"]),
                               mg_post=int(cfg["mg_post"]), mf_cells=int(cfg["mf_cells"]),
                               prec_reuse=float(cfg.get("prec_reuse", 0.0)))


def tune(gl, meshes: Sequence, params: Sequence, x0, linear_tol: float = 1e-4, tol: float = 1e-10,
         max_newton: int = 40, cache: Optional[str] = None, margin: float = 0.02) -> dict:
    """Tune for instances `meshes` with base Params `params` (one per mesh) from the start x0
    (concatenated node-major vectors).  With `cache` (a JSON path) earlier results for the
    same signature are reused and new ones stored."""
    import numpy as np

    precision = int(params[0].precision)
    key = signature(meshes, precision, extra=f"tol={linear_tol:g}/{tol:g}")
    store = {}
    if cache and os.path.exists(cache):
        with open(cache) as fh:
            store = json.load(fh)
        if key in store:
            out = dict(store[key])
            out["cached"] = True
            return out

    def measure(cfg):
        prms = [params_with(gl, p, cfg) for p in params]
        with gl.FemGL(list(meshes), prms) as f:
            if cfg["precond"] == "mg" and f.mg_levels == 0:
                return None  # multigrid does not apply: the block-Jacobi candidate covers it
            f.set_solution(np.asarray(x0))
            f.run(max_newton=max_newton, linear_tol=linear_tol, converge_acc=tol, allow_unconverged=True)
            f.set_solution(np.asarray(x0))
            f.sync()
            f.event_start()
            out = f.run(max_newton=max_newton, linear_tol=linear_tol, converge_acc=tol, allow_unconverged=True)
            ms = f.event_stop()
        return ms if bool(np.all(out["residual"] <= tol)) else None

    with gl.FemGL(list(meshes), [params_with(gl, p, DEFAULT) for p in params]) as f:
        multigrid = f.mg_levels > 0
    result = search(measure, margin=margin, multigrid=multigrid)
    result["signature"] = key
    if cache:
        store[key] = result
        tmp = cache + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(store, fh, indent=1)
        os.replace(tmp, cache)
    result["cached"] = False
    return result
