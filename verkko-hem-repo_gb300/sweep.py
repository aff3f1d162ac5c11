"""Sweeps larger than the device: many instances solved in waves of batched contexts.

A batched context keeps every instance's Jacobian blocks, Krylov bases and multigrid
hierarchy resident (in mixed precision with multigrid, tens of KB per mesh node), so a
phase-diagram sweep such as 256 slab instances of 16^3 to 48^3 cells (11.5M nodes) does not
fit one context.  ``solve_sweep`` measures the footprint on probe contexts of the largest
and the smallest instance (a constant per instance plus a slope per node), packs
consecutive instances into waves that fit the free device memory, solves each wave as one
batched context and returns the results in input order.
Instances are independent inside a context (per-instance reductions, GMRES, line search and
convergence); the preconditioner's storage and kernel shapes follow the context's total size
(FP16 coarse levels from 2000 nodes, warps per block row), so an instance's FP32 Krylov path
changes with its wave at rounding level and its converged state agrees to the Newton
tolerance.

The reference solves one configuration per program run (femgl/src/run.cc:157-258); the sweep
is the batched form of running it over many (T, p, thickness) points."""
import dataclasses
import time
from typing import Sequence

import numpy as np


def plan_waves(node_counts: Sequence[int], bytes_per_node: float, budget: float,
               bytes_per_instance: float = 0.0) -> list:
    """Consecutive groups of instance indices whose estimated footprint
    (bytes_per_instance + nodes x bytes_per_node per instance) stays within budget; raises
    ValueError for an instance that alone exceeds it."""
    waves, cur, used = [], [], 0.0
    for i, nn in enumerate(node_counts):
        need = bytes_per_instance + float(nn) * bytes_per_node
        if need > budget:
            raise ValueError(f"instance {i} ({nn} nodes, {need / 2**30:.2f} GiB) exceeds the budget "
                             f"of {budget / 2**30:.2f} GiB")
        if cur and used + need > budget:
            waves.append(cur)
            cur, used = [], 0.0
        cur.append(i)
        used += need
    if cur:
        waves.append(cur)
    return waves


def footprint(gl, meshes, params):
    """(bytes per node, bytes per instance) of a context, from probe contexts of the
    largest and the smallest instance: the hierarchy's small coarse levels, the Krylov
    bookkeeping and the per-instance tables weigh more per node on small meshes, so the
    footprint is fitted as a constant plus a per-node slope through the two probes."""
    sizes = [int(m.nn) for m in meshes]
    big, small = int(np.argmax(sizes)), int(np.argmin(sizes))
    with gl.FemGL(meshes[big], params[big]) as probe:
        b_big = float(probe.device_bytes)
    if sizes[small] == sizes[big]:
        return b_big / sizes[big], 0.0
    with gl.FemGL(meshes[small], params[small]) as probe:
        b_small = float(probe.device_bytes)
    slope = max(0.0, (b_big - b_small) / (sizes[big] - sizes[small]))
    const = max(0.0, b_small - slope * sizes[small])
    return slope, const


def finish_instance(gl, mesh, prm, x, *, max_newton: int = 40, linear_tol: float = 1e-4,
                    converge_acc: float = 1e-10) -> dict:
    """Finish one instance that a batched context handed off (its multigrid solve stalled twice)
    in a context of its own, from the state x it reached: first the same method with two pre-
    and two post-sweeps per level (handoff on again), then the same in FP64 (where a stall
    still finishes with block-Jacobi GMRES).  Returns newton_its, gmres_its, residual, free_energy, converged,
    solve_ms (device time), create_s, stage (the step that finished it) and x."""
    strong = {"mg_pre": max(2, int(prm.mg_pre)), "mg_post": max(2, int(prm.mg_post))}
    stages = [strong, dict(strong, precision=gl.FP64)]
    r = {"newton_its": 0, "gmres_its": 0, "solve_ms": 0.0, "create_s": 0.0}
    for k, change in enumerate(stages):
        last = k == len(stages) - 1
        t0 = time.perf_counter()
        with gl.FemGL(mesh, dataclasses.replace(prm, **change)) as g:
            r["create_s"] += time.perf_counter() - t0
            if not last:
                g.set_mg_handoff(True)
            g.set_solution(np.asarray(x, np.float64))
            g.sync()
            g.event_start()
            out = g.run(max_newton=max_newton, linear_tol=linear_tol, converge_acc=converge_acc,
                        allow_unconverged=True)
            r["solve_ms"] += g.event_stop()
            r["newton_its"] += int(out["newton_its"][0])
            r["gmres_its"] += int(out["gmres_its"][0])
            x = g.solution()
            if not last and bool(g.handed_off[0]):
                continue
            r.update({"residual": float(out["residual"][0]), "free_energy": float(g.free_energy()[0]),
                      "converged": bool(out["residual"][0] <= converge_acc), "stage": k, "x": x})
            return r
    raise AssertionError("unreachable")


def solve_sweep(gl, meshes, params, x0, *, max_newton: int = 40, linear_tol: float = 1e-4,
                converge_acc: float = 1e-10, budget: float | None = None, margin: float = 1.1,
                keep_solutions: bool = False, handoff: bool = True, log=None) -> dict:
    """Solve every instance (meshes[k], params[k], start x0[k]) to converge_acc, in waves.

    budget: device bytes a wave may take (default: 90 % of the free memory less 2 GiB).
    Returns per-instance arrays in input order (newton_its, gmres_its, residual,
    free_energy, converged, wave, handed_off) and per-wave timing: create_s (host plan,
    hierarchy and device setup), solve_ms (device time of the Newton solves, CUDA events),
    mg_fallbacks (multigrid solves of the wave finished with block-Jacobi).  With handoff (the
    default) an instance of a multi-instance wave whose multigrid solve stalls twice leaves the
    wave at the state it reached and is finished in a context of its own (finish_instance);
    its device time counts in its wave's solve_ms and in handoff_ms.  With keep_solutions the
    converged states come back as a list of arrays; log, when given, is called with one line
    per finished wave."""
    n = len(meshes)
    if not (len(params) == n and len(x0) == n):
        raise ValueError("meshes, params and x0 must have one entry per instance")
    sizes = [int(m.nn) for m in meshes]
    per_node, per_inst = footprint(gl, meshes, params)
    if budget is None:
        free, _ = gl.mem_info()
        budget = 0.9 * free - 2.0 * 2**30
    waves = plan_waves(sizes, per_node * margin, budget, per_inst * margin)
    res = {"newton_its": np.zeros(n, np.int32), "gmres_its": np.zeros(n, np.int32), "residual": np.zeros(n),
           "free_energy": np.zeros(n), "converged": np.zeros(n, bool), "wave": np.zeros(n, np.int32),
           "handed_off": np.zeros(n, bool)}
    sols = [None] * n if keep_solutions else None
    create_s, solve_ms, wave_bytes, fallbacks, handoff_ms = [], [], [], [], []
    for wi, w in enumerate(waves):
        t0 = time.perf_counter()
        f = gl.FemGL([meshes[i] for i in w], [params[i] for i in w])
        hand = handoff and len(w) > 1
        try:
            create_s.append(time.perf_counter() - t0)
            wave_bytes.append(f.device_bytes)
            if hand:
                f.set_mg_handoff(True)
            f.set_solution(np.concatenate([np.asarray(x0[i], np.float64) for i in w]))
            f.sync()
            f.event_start()
            out = f.run(max_newton=max_newton, linear_tol=linear_tol, converge_acc=converge_acc,
                        allow_unconverged=True)
            solve_ms.append(f.event_stop())
            F = f.free_energy()
            fallbacks.append(f.mg_fallbacks)
            handed = f.handed_off if hand else np.zeros(len(w), bool)
            x = f.solution() if (keep_solutions or handed.any()) else None
        finally:
            f.close()
        off = 0
        hand_ms = 0.0
        for j, i in enumerate(w):
            res["newton_its"][i] = out["newton_its"][j]
            res["gmres_its"][i] = out["gmres_its"][j]
            res["residual"][i] = out["residual"][j]
            res["free_energy"][i] = F[j]
            res["converged"][i] = out["residual"][j] <= converge_acc
            res["wave"][i] = wi
            xi = x[off:off + 18 * sizes[i]].copy() if x is not None else None
            if handed[j]:
                fin = finish_instance(gl, meshes[i], params[i], xi, max_newton=max_newton, linear_tol=linear_tol,
                                      converge_acc=converge_acc)
                res["newton_its"][i] += fin["newton_its"]
                res["gmres_its"][i] += fin["gmres_its"]
                res["residual"][i] = fin["residual"]
                res["free_energy"][i] = fin["free_energy"]
                res["converged"][i] = fin["converged"]
                res["handed_off"][i] = True
                hand_ms += fin["solve_ms"]
                create_s[-1] += fin["create_s"]
                xi = fin["x"]
            if keep_solutions:
                sols[i] = xi
            off += 18 * sizes[i]
        solve_ms[-1] += hand_ms
        handoff_ms.append(hand_ms)
        if log is not None:
            log(f"wave {wi}: {len(w)} instances, {sum(sizes[i] for i in w)} nodes, "
                f"{wave_bytes[-1] / 2**30:.1f} GiB, create {create_s[-1]:.1f} s, solve {solve_ms[-1]:.0f} ms"
                f" ({int(handed.sum())} handed off: {hand_ms:.0f} ms)")
    res.update({"waves": [len(w) for w in waves], "create_s": create_s, "solve_ms": solve_ms,
                "handoff_ms": handoff_ms, "wave_bytes": wave_bytes, "mg_fallbacks": fallbacks,
                "bytes_per_node": per_node, "bytes_per_instance": per_inst, "budget": budget})
    if keep_solutions:
        res["solutions"] = sols
    return res
