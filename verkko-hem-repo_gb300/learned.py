"""Learned Newton initial guess for slab phase-diagram sweeps.

Pipeline (no counterpart in the reference, which always starts from a uniform B phase,
femgl/src/setup_uniform_B-phase.cc:238-259):

1. converged states: batched mixed-precision Newton solves of seeded (t, p, D) slab
   instances from the uniform B phase (`generate`).  The uniform start has the symmetry of
   the slab (real, diagonal, u11 = u22); every converged state is then moved into one
   gauge (`canonical_gauge`): the global phase and spin rotations, exact symmetries of the
   functional, are fixed for the data rather than left to rounding;
2. training: the tcgen05 MLP of :class:`Surrogate` is fitted on per-node
   (features -> order parameter / bulk amplitude) pairs (`train`); the components that
   vanish in every training state (the symmetry zeros) are recorded;
3. inference: the network predicts every node of new instances and the symmetry zeros are
   set exactly (`guess`), so the start carries no error along the near-null phase and
   rotation directions, where Newton's linear solves converge slowly; plain Newton from
   that guess, and from the B phase for any instance whose residual stalls or that does
   not converge (`solve_learned`).

Features of a node at (x, y, z) of an instance (t, p, D) on a slab [-10, 10]^2 x
[-D/2, D/2]: (x/10, y/10, 2z/D, t, p/34, D/40).  Targets: the 18 components divided by
the bulk B-phase amplitude gap_B(p, t) * 0.577350269 of that instance.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

L_HALF = 10.0


def features(mesh, t: float, p: float, D: float) -> np.ndarray:
    xyz = np.asarray(mesh.xyz, np.float64)
    f = np.empty((xyz.shape[0], 6), np.float32)
    f[:, 0] = xyz[:, 0] / L_HALF
    f[:, 1] = xyz[:, 1] / L_HALF
    f[:, 2] = 2.0 * xyz[:, 2] / D
    f[:, 3] = t
    f[:, 4] = p / 34.0
    f[:, 5] = D / 40.0
    return f


def amplitude(gl, t: float, p: float) -> float:
    return gl.matep(p, t)["gap_B"] * float(np.float32(0.577350269))


@dataclasses.dataclass
class Instance:
    t: float
    p: float
    D: float
    n: int
    mesh: object


def sample(gl, count: int, seed: int, n_lo: int, n_hi: int):
    """Seeded (t, p, D, n) slab instances: t ~ U(0.3, 0.95), p ~ U(0, 34) (kept below 34),
    D ~ U(8, 40), n ~ U{n_lo..n_hi} cells per side."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        t = float(rng.uniform(0.3, 0.95))
        p = float(min(rng.uniform(0.0, 34.0), 34.0 - 1e-9))
        D = float(rng.uniform(8.0, 40.0))
        n = int(rng.integers(n_lo, n_hi + 1))
        m = gl.box_mesh([-L_HALF, -L_HALF, -D / 2], [L_HALF, L_HALF, D / 2], (n, n, n))
        out.append(Instance(t, p, D, n, m))
    return out


def bphase_starts(gl, insts, noise: float, seed: int):
    return [gl.bphase_guess(d.p, d.t, d.mesh.nn, noise=noise, seed=seed + k) for k, d in enumerate(insts)]


def solve(gl, insts, starts, precision, linear_tol=1e-4, tol=1e-10, max_newton=40, precond=None, gmres_max_iter=None):
    """One batched Newton run over the instances from the given starts.  Returns
    (solutions, stats, ms)."""
    pc = gl.PC_BLOCK_JACOBI if precond is None else precond
    kw = {} if gmres_max_iter is None else {"gmres_max_iter": int(gmres_max_iter)}
    prms = [gl.Params.from_matep(d.p, d.t, precision=precision, precond=pc, **kw) for d in insts]
    f = gl.FemGL([d.mesh for d in insts], prms)
    f.set_solution(np.concatenate(starts))
    f.sync()
    f.event_start()
    out = f.run(max_newton=max_newton, linear_tol=linear_tol, converge_acc=tol, allow_unconverged=True)
    ms = f.event_stop()
    x = f.solution()
    F = f.free_energy()
    f.close()
    offs = np.cumsum([0] + [18 * d.mesh.nn for d in insts])
    sols = [x[offs[k]:offs[k + 1]] for k in range(len(insts))]
    out["free_energy"] = F
    return sols, out, ms


def generate(gl, count: int, seed: int = 11, n_lo: int = 10, n_hi: int = 14, per_instance: int = 2048,
             noise: float = 0.0, precond=None, waves: bool = False):
    """Training pairs from `count` converged batched solves (from the uniform B phase
    unless noise > 0).  With waves, the instances are solved in device-sized waves of
    batched contexts (sweep.solve_sweep), for training sets larger than one context."""
    insts = sample(gl, count, seed, n_lo, n_hi)
    starts = bphase_starts(gl, insts, noise, seed * 1000)
    if waves:
        import importlib

        S = importlib.import_module(__package__ + ".sweep")
        pc = gl.PC_MULTIGRID if precond is None else precond
        prms = [gl.Params.from_matep(d.p, d.t, precision=gl.MIXED, precond=pc) for d in insts]
        r = S.solve_sweep(gl, [d.mesh for d in insts], prms, starts, keep_solutions=True)
        sols, ok, ms = r["solutions"], r["converged"], float(sum(r["solve_ms"]))
    else:
        sols, out, ms = solve(gl, insts, starts, gl.MIXED, precond=precond)
        ok = out["residual"] <= 1e-10
    rng = np.random.default_rng(seed)
    X, Y = [], []
    for d, x, good in zip(insts, sols, ok):
        if not good:
            continue
        f = features(d.mesh, d.t, d.p, d.D)
        y = (canonical_gauge(x).reshape(-1, 18) / amplitude(gl, d.t, d.p)).astype(np.float32)
        idx = rng.choice(f.shape[0], size=min(per_instance, f.shape[0]), replace=False)
        X.append(f[idx])
        Y.append(y[idx])
    return np.concatenate(X), np.concatenate(Y), {"instances": count, "solve_ms": ms, "converged": int(np.sum(ok))}


def canonical_gauge(x: np.ndarray, iters: int = 20) -> np.ndarray:
    """The state moved by the functional's exact symmetries (a global phase e^{i phi} and a
    spin rotation R acting on the spin index: A -> e^{i phi} R A) so that its mean order
    parameter is as close as possible to a positive multiple of the identity, i.e. the
    real diagonal form of the (distorted) B phase.  Converged states carry small arbitrary
    rotations: FP32 rounding in the linear solves is amplified along the near-null rotation
    directions.  (phi, R) maximise Re tr(e^{i phi} R C), C = sum over nodes of A, by
    alternating the phase and an orthogonal Procrustes rotation."""
    X = np.asarray(x, np.float64).reshape(-1, 18)
    A = (X[:, :9] + 1j * X[:, 9:]).reshape(-1, 3, 3)
    C = A.sum(axis=0)
    R = np.eye(3)
    phi = 0.0
    for _ in range(iters):
        phi = -float(np.angle(np.trace(R @ C)))
        U, _, Vt = np.linalg.svd(np.real(np.exp(1j * phi) * C))
        D = np.diag([1.0, 1.0, np.sign(np.linalg.det(Vt.T @ U.T))])
        R = Vt.T @ D @ U.T
    Al = np.exp(1j * phi) * np.einsum("ij,njk->nik", R, A)
    return np.concatenate([Al.real.reshape(-1, 9), Al.imag.reshape(-1, 9)], axis=1).reshape(-1)


def symmetry_zeros(Y, rel: float = 1e-4) -> np.ndarray:
    """Output mask: 0 for the components that vanish (below rel times the largest target)
    in every training state, 1 elsewhere."""
    amax = np.abs(Y).max(axis=0)
    return (amax > rel * amax.max()).astype(np.float32)


def train(gl, X, Y, steps: int = 1500, batch: int = 4096, lr: float = 1e-3, seed: int = 0):
    """Fits a Surrogate on (X, Y); its `out_mask` attribute holds the symmetry zeros."""
    s = gl.Surrogate(seed=seed)
    mask = symmetry_zeros(Y)
    t0 = time.perf_counter()
    loss = s.train(X, Y * mask, steps=steps, batch=batch, lr=lr, seed=seed)
    s.out_mask = mask
    return s, {"loss": loss, "train_s": time.perf_counter() - t0, "steps": steps, "batch": batch,
               "rows": int(X.shape[0]), "components_kept": int(mask.sum())}


def guess(gl, surrogate, insts):
    """Surrogate initial guesses (FP64 node-major vectors) for the instances, with the
    symmetry zeros of the training data set exactly."""
    mask = getattr(surrogate, "out_mask", None)
    out = []
    for d in insts:
        y = surrogate.predict(features(d.mesh, d.t, d.p, d.D)).astype(np.float64)
        if mask is not None:
            y *= mask
        out.append((y * amplitude(gl, d.t, d.p)).ravel())
    return out


# GMRES iterations per Newton step allowed from a learned start: the learned state's
# remaining error lies largely along near-symmetry (phase, rotation) directions, where a
# linear solve can stall; a stalled instance is re-solved from the B phase instead
LEARNED_GMRES_CAP = 300


def solve_learned(gl, surrogate, insts, precision, linear_tol=1e-4, tol=1e-10, max_newton=40, noise_fallback=0.05,
                  fallback_seed=0, precond=None, gmres_cap=LEARNED_GMRES_CAP):
    """Newton from the surrogate; instances that do not reach tol (their residual or a
    linear solve stalls) are re-solved from the B phase.  Returns (solutions, per-instance
    stats dict, total ms, info)."""
    t0 = time.perf_counter()
    starts = guess(gl, surrogate, insts)
    t_guess = (time.perf_counter() - t0) * 1000.0
    sols, out, ms = solve(gl, insts, starts, precision, linear_tol, tol, max_newton, precond, gmres_cap)
    failed = [k for k in range(len(insts)) if not (out["residual"][k] <= tol)]
    fb_ms = 0.0
    if failed:
        sub = [insts[k] for k in failed]
        s2, o2, fb_ms = solve(gl, sub, bphase_starts(gl, sub, noise_fallback, fallback_seed), precision, linear_tol, tol,
                              max_newton, precond)
        for j, k in enumerate(failed):
            sols[k] = s2[j]
            out["newton_its"][k] += o2["newton_its"][j]
            out["residual"][k] = o2["residual"][j]
            out["free_energy"][k] = o2["free_energy"][j]
    return sols, out, ms + fb_ms + t_guess, {"fallbacks": len(failed), "guess_ms": t_guess}
