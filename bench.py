"""Benchmark of the femgl Newton hot path on one GB300.

Workload (the femgl 3D configuration the metric is quoted on): cube [-10, 10]^3
(L = 20 xi0), 32^3 Q1 hexahedra, matep coefficients at T = 0.6 Tc, p = 20 bar with
strong-coupling corrections, pair-breaking A_{mu z} = 0 on the z faces, free
elsewhere, start = B phase + 0.05 N(0,1) per dof (seed 2).  Nd = 646,866 dofs,
nnzb = 912,673 18x18 blocks.

One step = one complete Newton solve from that start to ||F||_2 < 1e-10 (the
reference's run() loop), inputs resident in HBM.  value = solves/s of the mixed
solver (FP32 Jacobian + FP32 GMRES, FP64 residual/line search); the plain FP64 GPU
Newton is measured in the same run and reported beside it, together with assembly
GDOF/s.  e2e = the same solves through the C ABI with the start vector copied in
from host memory and the solution copied out every step.

--impl reference times the CPU implementation instead (see cpu_reference()).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

P_BAR, T_RED, HALF, NCELL, NOISE, SEED = 20.0, 0.6, 10.0, 32, 0.05, 2
TOL = 1e-10
# DRAM bytes of one matrix-free apply (k_mf_cell + k_mf_gather in the y = J z form) on this
# workload, from ncu captures of the two kernels on the 32^3 cube (`--ncu-case 32`; cold caches:
# the cell results the gather reads come from DRAM there, from L2 in the live solve)
MF_NCU_TRAFFIC = 7.073536e6 + 0.0 + 2.2761216e7
# FP32 operations of one matrix-free apply per cell: the closed-form Hessian-vector product at
# 8 points, regrouped as C Re(A) + D Im(A) + E Re(F) + G Im(F) (about 1,500 per point: the
# products A F^T and F A^+, the state-only A A^T and A A^+, four complex-by-real 3x3 products)
# plus the interpolation of state and direction, the gradient terms and the transposed
# contraction
MF_FLOP_PER_CELL = 8 * 1500 + 4500
METRIC = "GL solves/s at ||F||<1e-10 (femgl 3D, 32^3 Q1, T=0.6Tc, p=20bar)"
WORKLOAD = "femgl 3D cube L=20, 32^3 Q1 cells, matep(p=20 bar, t=0.6, SCC), z-face pair breaking, B-phase+0.05N(0,1) seed 2"


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", "0", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 2 + i and s[2 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def problem(gl):
    m = gl.cube_mesh(HALF, NCELL)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=NOISE, seed=SEED)
    return m, x0


def solve_once(f, x0, linear_tol):
    if callable(x0):
        x0 = x0()  # learned start: network inference happens inside the timed step
    f.set_solution(x0)
    return f.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL)


def batch_instances(gl, count, seed=4):
    """Seeded sample of the batched phase-diagram sweep: T/Tc ~ U(0.3, 0.95),
    p ~ U(0, 34) bar (kept below 34, where the coefficient tables end), slab thickness
    D ~ U(8, 40) xi0 across z (pair-breaking faces), lateral 20 xi0, n^3 Q1 cells with
    n ~ U{16..48}; start = B phase + 0.05 N(0,1)."""
    rng = np.random.default_rng(seed)
    pts = []
    for _ in range(count):
        t = float(rng.uniform(0.3, 0.95))
        p = float(min(rng.uniform(0.0, 34.0), 34.0 - 1e-9))
        D = float(rng.uniform(8.0, 40.0))
        n = int(rng.integers(16, 49))
        pts.append((t, p, D, n))

    def make(k):
        t, p, D, n = pts[k]
        m = gl.box_mesh([-10.0, -10.0, -D / 2], [10.0, 10.0, D / 2], (n, n, n))
        x0 = gl.bphase_guess(p, t, m.nn, noise=NOISE, seed=1000 + k)
        return {"t": t, "p": p, "D": D, "n": n, "mesh": m, "x0": x0}

    # the meshers release the interpreter lock: build the instances on the host threads (the
    # library is loaded and its signatures set before the threads start)
    from concurrent.futures import ThreadPoolExecutor
    gl.lib()
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        return list(ex.map(make, range(count)))


def batched_leg(gl, count, linear_tol, sur=None, precond=None, cfg=None):
    """Batched mixed solve of `count` instances in one context (from the B phase and, with
    a surrogate, from its guess) vs FP64 GPU Newton solving them one at a time from the B
    phase, with the same preconditioner and with the plain method (block-Jacobi GMRES);
    all to ||F|| < 1e-10 per instance."""
    inst = batch_instances(gl, count)
    meshes = [d["mesh"] for d in inst]
    x0 = np.concatenate([d["x0"] for d in inst])
    pc = gl.PC_BLOCK_JACOBI if precond is None else precond
    prm_m = [gl.Params.from_matep(d["p"], d["t"], precision=gl.MIXED, precond=pc) for d in inst]
    if cfg is not None:  # the configuration the autotuner chose for the headline workload
        AT = importlib.import_module("verkko-hem-repo_gb300.autotune")
        prm_m = [AT.params_with(gl, p, cfg) for p in prm_m]
    f = gl.FemGL(meshes, prm_m)
    f.set_solution(x0)
    f.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL)  # warm-up
    f.set_solution(x0)
    f.sync()
    f.event_start()
    out = f.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL)
    ms_batch = f.event_stop()
    F_b = f.free_energy()
    f.close()
    ms_seq = 0.0
    F_s = []
    its_s = []
    for d in inst:
        prm = gl.Params.from_matep(d["p"], d["t"], precision=gl.FP64, precond=pc)
        g = gl.FemGL(d["mesh"], prm)
        g.set_solution(d["x0"])
        g.sync()
        g.event_start()
        o = g.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL)
        ms_seq += g.event_stop()
        F_s.append(g.free_energy()[0])
        its_s.append(int(o["newton_its"][0]))
        g.close()
    F_s = np.array(F_s)
    # the plain FP64 GPU Newton (block-Jacobi GMRES, the method without multigrid) on the
    # same instances, one at a time
    ms_plain = 0.0
    for d in inst:
        prm = gl.Params.from_matep(d["p"], d["t"], precision=gl.FP64, precond=gl.PC_BLOCK_JACOBI)
        g = gl.FemGL(d["mesh"], prm)
        g.set_solution(d["x0"])
        g.sync()
        g.event_start()
        g.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL)
        ms_plain += g.event_stop()
        g.close()
    learned = None
    if sur is not None:
        L = importlib.import_module("verkko-hem-repo_gb300.learned")
        li = [L.Instance(d["t"], d["p"], d["D"], d["n"], d["mesh"]) for d in inst]
        L.solve_learned(gl, sur, li, gl.MIXED, linear_tol, precond=pc)  # warm-up
        _, ol, ms_l, finfo = L.solve_learned(gl, sur, li, gl.MIXED, linear_tol, precond=pc)
        learned = {"mixed_batched_learned_solves_per_s": count / (ms_l / 1000.0),
                   "speedup_vs_fp64_sequential": ms_seq / ms_l, "speedup_vs_plain_fp64": ms_plain / ms_l,
                   "newton_its": ol["newton_its"].tolist(),
                   "max_free_energy_rel_diff_vs_fp64": float(np.max(np.abs(ol["free_energy"] - F_s) / np.abs(F_s))),
                   "all_converged": bool(np.all(ol["residual"] <= TOL)), "fallbacks": finfo["fallbacks"]}
    return {"instances": count, "learned": learned, "total_dofs": int(sum(18 * m.nn for m in meshes)),
            "mixed_batched_solves_per_s": count / (ms_batch / 1000.0),
            "fp64_sequential_solves_per_s": count / (ms_seq / 1000.0),
            "plain_fp64_sequential_solves_per_s": count / (ms_plain / 1000.0),
            "speedup": ms_seq / ms_batch, "speedup_vs_plain_fp64": ms_plain / ms_batch,
            "all_converged": bool(out["converged"]),
            "max_final_residual": float(out["residual"].max()),
            "max_free_energy_rel_diff_vs_fp64": float(np.max(np.abs(F_b - F_s) / np.abs(F_s))),
            "newton_its_batched": out["newton_its"].tolist(), "newton_its_fp64": its_s,
            "sample": "seeded (seed 4) instances of the sweep: T/Tc~U(0.3,0.95), p~U(0,34), D~U(8,40), n~U{16..48}"}


def time_mode(gl, m, x0, precision, steps, warmup, linear_tol, kernel_timing=False, flush=None, precond=None,
              cfg=None, prepare=None, **prm_kw):
    prm = gl.Params.from_matep(P_BAR, T_RED, precision=precision,
                               precond=gl.PC_BLOCK_JACOBI if precond is None else precond, **prm_kw)
    if cfg is not None:
        prm = importlib.import_module("verkko-hem-repo_gb300.autotune").params_with(gl, prm, cfg)
    f = gl.FemGL(m, prm)
    if prepare is not None:
        prepare(f)
    out = None
    for _ in range(warmup):
        out = solve_once(f, x0, linear_tol)
    f.timers(reset=True)
    f.kernel_timing(1 if kernel_timing else 0, reset=True)  # bit 0: SpMV launches only
    launches0 = f.launch_count
    ms_steps = []
    stats = []
    for _ in range(steps):
        if flush is not None:
            flush()
        f.sync()
        f.event_start()
        out = solve_once(f, x0, linear_tol)
        ms_steps.append(f.event_stop())
        stats.append(out)
    kms, kn = f.kernel_timing(False)
    phases = f.timers()
    launches = f.launch_count - launches0
    mg = {"levels": f.mg_levels, "fallbacks": f.mg_fallbacks}
    x = f.solution()
    F = float(f.free_energy()[0])
    # assembly alone (J + R at a fresh state: set_solution drops the residual that a line
    # search left behind), timed call by call
    xs = x0() if callable(x0) else x0
    f.set_solution(xs)
    f.assemble_system()
    na = 5
    asm_ms = 0.0
    for _ in range(na):
        f.set_solution(xs)
        f.event_start()
        f.assemble_system()
        asm_ms += f.event_stop() / na
    f.close()
    return {"ms": ms_steps, "out": stats[-1], "kernel_ms": kms, "kernel_n": kn, "phases": phases,
            "launches": launches, "x": x, "F": F, "asm_ms": asm_ms, "mg": mg}


def e2e_mode(gl, m, x0, precision, steps, linear_tol, precond=None, cfg=None):
    prm = gl.Params.from_matep(P_BAR, T_RED, precision=precision,
                               precond=gl.PC_BLOCK_JACOBI if precond is None else precond)
    if cfg is not None:
        prm = importlib.import_module("verkko-hem-repo_gb300.autotune").params_with(gl, prm, cfg)
    f = gl.FemGL(m, prm)
    # the step's input and output live in page-locked host memory
    x_in = gl.pinned_array(f.n_dofs)
    x_out = gl.pinned_array(f.n_dofs)
    if callable(x0):
        start = x0  # the learned start: network inference on host inputs gives the vector
    else:
        x_in[:] = x0
        start = lambda: x_in  # noqa: E731
    solve_once(f, start(), linear_tol)
    t0 = time.perf_counter()
    for _ in range(steps):
        f.set_solution(start())  # host -> device
        f.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL)
        f.solution(out=x_out)  # device -> host
    dt = time.perf_counter() - t0
    xo = np.array(x_out)
    f.close()
    return steps / dt, xo


def oracle_problem():
    """The benchmark workload built from the oracle alone (no part of the CUDA library):
    the oracle's mesher, the reference's matep values (its own compiled matep where the
    reference tree was built here, else the committed table of that matep's outputs), the
    seeded B-phase start and the oracle's FP64 condensed system.  Returns (system, x0)."""
    from oracle import gl as ogl
    from oracle import mesh as om

    ogl.build()
    m = om.box_mesh([-HALF] * 3, [HALF] * 3, (NCELL,) * 3)
    mp = ogl.matep(P_BAR, T_RED)
    coef = ogl.coef_vector(mp["alpha"], [mp[f"beta{i}"] for i in range(1, 6)])
    x0 = ogl.bphase_guess(mp["gap_B"], m.nn, NOISE, SEED)
    return ogl.System(m, coef), x0


def cpu_solves(sysr, x0, linear_tol, budget_s, min_solves=1):
    """Complete FP64 Newton solves of the workload on all host cores with the oracle's C
    restatement: OpenMP assembly and residual, block-Jacobi GMRES(50) to linear_tol * |rhs|
    (the reference uses FGMRES with Trilinos ML AMG, femgl/src/solve.cc:130-174, which
    does not exist here), the reference's damped line search (iteration.cc:170-206) and
    stop rule (run.cc:234).  Solves repeat while the elapsed time stays below budget_s.
    Returns (seconds per solve, solves, Newton its, GMRES its, threads, final |F|)."""
    from oracle import gl as ogl

    times, hist, x = [], None, None
    while len(times) < min_solves or sum(times) < budget_s:
        t0 = time.perf_counter()
        x, hist = ogl.newton(sysr, x0, tol=TOL, max_iter=40, linear_tol=linear_tol)
        times.append(time.perf_counter() - t0)
        if sum(times) + times[-1] > budget_s:
            break
    cpu_solves.last_x = x
    return (float(np.mean(times)), len(times), len(hist), sum(h["linear_its"] for h in hist),
            ogl.lib().orc_num_threads(), hist[-1]["res"])


def err_vs_oracle(sysr, x_oracle, x_gpu, F_gpu):
    """The GPU's converged state against the oracle's converged FP64 solve of the same
    workload: max |x - x_oracle| / max |x_oracle|, the free energies, and the oracle's own
    FP64 residual norm and free energy at the GPU's state."""
    from oracle import gl as ogl

    R_o, F_o = sysr.residual(x_gpu)
    _, F_ref = sysr.residual(x_oracle)
    xa, _, _ = ogl.gauge_align(x_gpu, x_oracle)
    return {"x_max_rel": float(np.abs(xa - x_oracle).max() / np.abs(x_oracle).max()),
            "x_max_rel_unaligned": float(np.abs(x_gpu - x_oracle).max() / np.abs(x_oracle).max()),
            "x_note": "after the exact global phase and spin rotation that best align the two states (the "
                      "functional's symmetries, along which the Jacobian is singular at a solution)",
            "F_rel": abs(F_gpu - F_ref) / abs(F_ref),
            "oracle_residual_at_gpu_state": float(np.linalg.norm(R_o)),
            "oracle_F_at_gpu_state_rel": abs(F_gpu - F_o) / abs(F_o),
            "oracle_solve": "FP64 Newton, block-Jacobi GMRES(50) to the same linear tolerance"}


def cpu_port_baseline(linear_tol):
    """Returns (the oracle system, the oracle's converged x, the cpu_baseline entry)."""
    sysr, x0 = oracle_problem()
    sysr.assemble(sysr.distribute(x0), want_J=False)  # warm-up of the timed object
    dt, ns, nn, gi, thr, res = cpu_solves(sysr, x0, linear_tol, budget_s=20.0)
    return sysr, cpu_solves.last_x, {"value": 1.0 / dt, "unit": "solves/s", "cores": thr, "kind": "port",
            "method": "block-Jacobi GMRES(50) port; compare with this line's mixed_block_jacobi entry (same method "
                      "on the GPU) for the hardware gap alone",
            "sample": f"{ns} complete FP64 Newton solve(s) of the same 32^3 workload on {thr} host threads with "
                      f"the oracle port ({nn} Newton its, {gi} block-Jacobi GMRES(50) its, final |F| {res:.2e}, "
                      f"{dt:.1f} s per solve)"}


def reference_kernels_leg(sysr, x0, threads):
    """The reference's own cell loop (assemble.cc:188-280 over its cell_mat_vec kernels,
    compiled unmodified) timed on 64 cells of the workload spread over the mesh: 8 cells
    on 1 thread, all 64 on every host thread; extrapolated to the mesh's 32,768 cells."""
    from oracle import gl as ogl

    if ogl.ref() is None:
        return {"unavailable": "the reference's kernels are compiled only where the reference tree is present, "
                              "which is not this host"}
    m = sysr.m
    x = sysr.distribute(x0)
    pick = np.linspace(0, m.nc - 1, 64).astype(np.int64)
    xc = x.reshape(-1, 18)[m.cells[pick]]  # [64][8][18]
    h = m.xyz[m.cells[0, 7]] - m.xyz[m.cells[0, 0]]
    c = sysr.coef
    coef9 = np.array([c[0], 0.5 * c[1], 0.5 * c[1], c[2], *c[3:8]])  # K2 = K3 = (K2+K3)/2
    t1, K1, _ = ogl.time_reference_cells(h, xc[:8], coef9, 1)
    tn, Kn, _ = ogl.time_reference_cells(h, xc, coef9, threads)
    if not np.array_equal(K1, Kn[:8]):
        raise RuntimeError("threaded reference cell loop differs from the serial one")
    nd = 18 * m.nn
    s1 = t1 / 8 * m.nc
    sn = tn / 64 * m.nc
    return {"kind": "reference", "cells_timed": {"1_thread": 8, f"{threads}_threads": 64},
            "s_per_cell_1_thread": t1 / 8, "assembly_s_1_thread_extrapolated": s1,
            "assembly_s_all_threads_extrapolated": sn, "threads": threads,
            "assembly_gdofs_1_thread_extrapolated": nd / s1 / 1e9,
            "assembly_gdofs_all_threads_extrapolated": nd / sn / 1e9,
            "note": "extrapolated: (cells timed) / (time) scaled to all 32,768 cells of one assembly"}


def bench_config(linear_tol):
    """The workload keys both arms report (the solver each arm uses is under 'solver')."""
    return {"workload": WORKLOAD, "n_dofs": 646866, "nnzb": 912673, "n_cells": NCELL ** 3, "converge_acc": TOL,
            "linear_tol": linear_tol,
            "l2": "inputs > L2 (the FP32 block matrix alone is 1.18 GB); the GPU arm also writes a 256 MB buffer "
                  "between timed steps"}


def make_parser():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--linear-tol", type=float, default=1e-4)
    ap.add_argument("--ncu-case", type=int, default=0,
                    help="profiling case: one mixed assembly + 30 GMRES iterations on an N^3 cube, no timing")
    ap.add_argument("--fp64", action="store_true", help="with --ncu-case / --ncu-solve: FP64 instead of mixed")
    ap.add_argument("--ncu-solve", type=int, default=0,
                    help="profiling case: one complete Newton solve of the N^3 cube (--precond), no timing")
    ap.add_argument("--prec-reuse", type=float, default=0.0,
                    help="with --ncu-solve: keep the preconditioner while the last step is below this")
    ap.add_argument("--batch", type=int, default=8, help="instances in the batched leg (0 = skip)")
    ap.add_argument("--config3", action="store_true", help="only the refined 64^3 mixed-vs-FP64 leg")
    ap.add_argument("--config4", type=int, default=0,
                    help="only the full-scale batched sweep: this many seeded slab instances, in waves")
    ap.add_argument("--config5", type=int, nargs=2, default=None, metavar=("N_TRAIN", "N_TEST"),
                    help="only the learned-start leg at scale: train on N_TRAIN converged states, test on N_TEST "
                         "held-out 48^3 slab instances")
    ap.add_argument("--no-learned", dest="learned", action="store_false", help="skip the learned initial guess")
    ap.add_argument("--ncu-mlp", type=int, default=0, help="profiling case: surrogate forward on N points + one gradient")
    ap.add_argument("--precond", default="mg", choices=["mg", "bj"],
                    help="preconditioner of every GPU leg: geometric multigrid (default) or block-Jacobi")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the autotuner (the headline then uses the default configuration)")
    ap.add_argument("--headline-start", default="auto", choices=["auto", "bphase", "learned"],
                    help="start of the headline solves: the learned guess where it solves faster than the B phase "
                         "(auto), or either one (the other start is reported beside it)")
    return ap


def main():
    args = make_parser().parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.ncu_case:
        return ncu_case(args.ncu_case, args.fp64)
    if args.ncu_solve:
        return ncu_solve(args.ncu_solve, args.fp64, args.precond, args.prec_reuse)
    if args.ncu_mlp:
        gl = importlib.import_module("verkko-hem-repo_gb300")
        gl.build()
        rng = np.random.default_rng(0)
        X = rng.uniform(-1, 1, (args.ncu_mlp, 6)).astype(np.float32)
        with gl.Surrogate(seed=1) as sm:
            y = sm.predict(X)
            T = rng.standard_normal((min(args.ncu_mlp, 16384), 18)).astype(np.float32)
            loss, _ = sm.gradient(X[: T.shape[0]], T)
        print(json.dumps({"ncu_mlp": args.ncu_mlp, "out_norm": float(np.linalg.norm(y)), "loss": loss}))
        return 0
    if args.config3:
        gl = importlib.import_module("verkko-hem-repo_gb300")
        gl.build()
        print(json.dumps({"config3": config3_leg(gl, args.linear_tol)}))
        return 0
    if args.config4:
        gl = importlib.import_module("verkko-hem-repo_gb300")
        gl.build()
        print(json.dumps({"config4": config4_leg(gl, args.config4, args.linear_tol)}))
        return 0
    if args.config5:
        gl = importlib.import_module("verkko-hem-repo_gb300")
        gl.build()
        print(json.dumps({"config5": config5_leg(gl, args.config5[0], args.config5[1], args.linear_tol)}))
        return 0
    if args.impl == "reference":
        return reference_arm(args, rank)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1 and rank != 0:
        # one replica per GPU is the multi-GPU form of this path (instances are independent,
        # no exchange); this build measures and reports the single-GPU replica on rank 0
        return 0
    gl = importlib.import_module("verkko-hem-repo_gb300")
    gl.build()
    m, x0 = problem(gl)
    pk = peaks()
    hbm = float(pk.get("hbm_gbs", 6800.0))

    import ctypes

    # L2 flush buffer (256 MB > 129 MB L2): written between timed steps
    flush_buf = None
    try:
        import torch

        if torch.cuda.is_available():
            flush_buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    except Exception:
        flush_buf = None

    def flush():
        if flush_buf is not None:
            flush_buf.fill_(1.0)
            import torch

            torch.cuda.synchronize()

    pc = gl.PC_MULTIGRID if args.precond == "mg" else gl.PC_BLOCK_JACOBI
    # learned initial guess: trained once, before any timing, on converged states of
    # seeded slab instances (none of them is the benchmark instance)
    sur, learn_info = None, None
    if args.learned:
        L = importlib.import_module("verkko-hem-repo_gb300.learned")
        t0 = time.perf_counter()
        Xtr, Ytr, ginfo = L.generate(gl, 32, seed=11, n_lo=10, n_hi=14, per_instance=2048, precond=pc)
        t_gen = time.perf_counter() - t0
        sur, tinfo = L.train(gl, Xtr, Ytr, steps=3000, batch=4096, lr=1e-3, seed=0)
        inst2 = L.Instance(T_RED, P_BAR, 2 * HALF, NCELL, m)
        learned_x0 = lambda: L.guess(gl, sur, [inst2])[0]  # noqa: E731
        learn_info = {"train_states": ginfo["converged"], "train_rows": tinfo["rows"], "train_steps": tinfo["steps"],
                      "train_loss": tinfo["loss"], "data_generation_s": t_gen, "training_s": tinfo["train_s"],
                      "mlp_launches": sur.launch_count,
                      "note": "trained once before timing on 32 seeded slab instances (10^3-14^3 cells), "
                              "not including the benchmark instance"}
    fp64 = time_mode(gl, m, x0, gl.FP64, max(1, args.steps // 2), 1, args.linear_tol, kernel_timing=True, flush=flush,
                     precond=pc)
    # block-Jacobi beside multigrid (same start, same precision)
    bj = time_mode(gl, m, x0, gl.MIXED, max(1, args.steps // 2), 1, args.linear_tol, flush=flush,
                   precond=gl.PC_BLOCK_JACOBI) if pc != gl.PC_BLOCK_JACOBI else None
    # the autotuner picks preconditioner, restart, multigrid sweeps, the matrix-free
    # operator's cell batch and the preconditioner-reuse threshold for this workload, once
    # per start (complete solves timed before the timed region)
    AT = importlib.import_module("verkko-hem-repo_gb300.autotune")
    base_prm = [gl.Params.from_matep(P_BAR, T_RED, precision=gl.MIXED)]
    tuned = tuned_l = None
    if args.autotune:
        t0 = time.perf_counter()
        tuned = AT.tune(gl, [m], base_prm, x0, args.linear_tol, TOL)
        tuned["tuning_s"] = time.perf_counter() - t0
        if sur is not None:
            t0 = time.perf_counter()
            tuned_l = AT.tune(gl, [m], base_prm, learned_x0(), args.linear_tol, TOL)
            tuned_l["tuning_s"] = time.perf_counter() - t0
    cfg_b = tuned["config"] if tuned else None
    cfg_l = tuned_l["config"] if tuned_l else cfg_b
    # the learned start, network inference inside every timed solve, with its own tuning
    alt = time_mode(gl, m, learned_x0, gl.MIXED, max(1, args.steps // 2), 1, args.linear_tol, flush=flush,
                    precond=pc, cfg=cfg_l) if sur is not None else None
    # the headline start: the learned guess when it solves faster (auto), or as asked
    ref_b = time_mode(gl, m, x0, gl.MIXED, max(1, args.steps // 2), 1, args.linear_tol, flush=flush,
                      precond=pc, cfg=cfg_b)
    if args.headline_start == "auto" and alt is not None:
        use_learned = float(np.mean(alt["ms"])) < float(np.mean(ref_b["ms"]))
    else:
        use_learned = alt is not None and args.headline_start == "learned"
    head_x0 = learned_x0 if use_learned else x0
    head_cfg = cfg_l if use_learned else cfg_b
    with ClockSampler() as clk:
        mixed = time_mode(gl, m, head_x0, gl.MIXED, args.steps, args.warmup, args.linear_tol, kernel_timing=True,
                          flush=flush, precond=pc, cfg=head_cfg)
    # the same solve with the kernels in plain stream order (programmatic dependent launch off)
    gl.set_launch_mode(False)
    try:
        plain = time_mode(gl, m, head_x0, gl.MIXED, max(1, args.steps // 2), 1, args.linear_tol, flush=flush,
                          precond=pc, cfg=head_cfg)
    finally:
        gl.set_launch_mode(True)
    # the small coarse levels as one cooperative launch per V-cycle instead of separate launches
    fused = time_mode(gl, m, head_x0, gl.MIXED, max(1, args.steps // 2), 1, args.linear_tol, flush=flush,
                      precond=pc, cfg=head_cfg, mg_small_fuse=1)
    # the V-cycle's tail (levels of at most 160 nodes and the dense solve) as one cluster launch
    tail = time_mode(gl, m, head_x0, gl.MIXED, max(1, args.steps // 2), 1, args.linear_tol, flush=flush,
                     precond=pc, cfg=head_cfg, mg_small_fuse=2)
    # GMRES with a reorthogonalized Gram-Schmidt (one more pass over the basis) beside the
    # default single projection
    cgs2 = time_mode(gl, m, head_x0, gl.MIXED, max(1, args.steps // 2), 1, args.linear_tol, flush=flush,
                     precond=pc, cfg=head_cfg, prepare=lambda f: f.set_reorthogonalization(True))
    e2e_val, x_e2e = e2e_mode(gl, m, head_x0, gl.MIXED, max(1, args.steps), args.linear_tol, precond=pc, cfg=head_cfg)
    batched = batched_leg(gl, args.batch, args.linear_tol, sur, precond=pc, cfg=head_cfg) if args.batch > 0 else None

    ms_step = float(np.mean(mixed["ms"]))
    value = 1000.0 / ms_step
    nd = 18 * m.nn
    nnzb = 912673
    # the Krylov operator of the mixed path: J z applied matrix-free at the state
    # (k_mf_cell + k_mf_gather, two launches per apply); algorithmic bytes per apply: the FP32
    # state and z in, y out, cell connectivity, geometry and instance id.  It is bound by FP32
    # issue, not HBM: the fp32 entry gives its arithmetic rate against the CUDA-core peak at
    # the SM clock sampled during the run
    mf_bytes = 3 * nd * 4 + m.nc * (8 * 4 + 16 + 4)
    n_mf = mixed["kernel_n"]["spmv"] // 2
    mf_ms = mixed["kernel_ms"]["spmv"] / max(1, n_mf)
    achieved = mf_bytes / (mf_ms * 1e-3) / 1e9 if n_mf else None
    mf_flop = m.nc * MF_FLOP_PER_CELL
    sm_mhz = clk.summary().get("sm_mhz") or 2070.0
    n_sm = 152
    try:
        import torch

        n_sm = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    fp32_peak = n_sm * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s: SMs x 128 FP32 lanes x FMA
    mf_tflops = mf_flop / (mf_ms * 1e-3) / 1e12 if n_mf else None
    # the FP64 path's operator: the assembled block SpMV, timed in the FP64 leg
    spmv_bytes = nnzb * (324 * 8 + 4) + (m.nn + 1) * 4 + 2 * nd * 8
    n_spmv = fp64["kernel_n"]["spmv"]
    spmv_ms = fp64["kernel_ms"]["spmv"] / max(1, n_spmv)
    spmv_gbs = spmv_bytes / (spmv_ms * 1e-3) / 1e9 if n_spmv else None
    asm_bytes = nnzb * 324 * 4 + m.nc * 32 + 2 * nd * 8
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 Jacobian/GMRES + f64 residual (bf16 tensor-core MLP for the start)",
        "data": "synthetic (seeded B-phase + Gaussian noise start; no dataset)",
        "config": bench_config(args.linear_tol),
        "solver": {"mode": "mixed+learned" if use_learned else "mixed",
                   "precond": ("geometric multigrid: Galerkin coarse levels, l1 block-Jacobi smoothing, "
                               "flexible GMRES") if (head_cfg or {"precond": "mg" if pc == gl.PC_MULTIGRID else "bj"})[
                                   "precond"] == "mg" else "block-Jacobi, GMRES",
                   "solver_config": head_cfg, "mg_levels": mixed["mg"]["levels"], "gmres_restart": 50},
        "newton_its": int(mixed["out"]["newton_its"][0]),
        "gmres_its": int(mixed["out"]["gmres_its"][0]),
        "final_residual": float(mixed["out"]["residual"][0]),
        "final_residual_kind": "FP64 residual at the converged state (the stop test)",
        "final_residual_line_search": float(mixed["out"]["residual_line_search"][0]),
        "free_energy": mixed["F"],
        "fp64": {"solves_per_s": 1000.0 / float(np.mean(fp64["ms"])), "ms_per_solve": float(np.mean(fp64["ms"])),
                 "newton_its": int(fp64["out"]["newton_its"][0]), "gmres_its": int(fp64["out"]["gmres_its"][0]),
                 "free_energy": fp64["F"], "assembly_ms": fp64["asm_ms"], "assembly_gdofs": nd / fp64["asm_ms"] / 1e6},
        "mixed_block_jacobi": None if bj is None else {
            "solves_per_s": 1000.0 / float(np.mean(bj["ms"])), "ms_per_solve": float(np.mean(bj["ms"])),
            "newton_its": int(bj["out"]["newton_its"][0]), "gmres_its": int(bj["out"]["gmres_its"][0]),
            "free_energy": bj["F"]},
        "mg_fallbacks": mixed["mg"]["fallbacks"],
        "launch_mode": {"programmatic_ms_per_solve": ms_step, "plain_ms_per_solve": float(np.mean(plain["ms"])),
                        "note": "programmatic dependent launch (the default) against plain stream order"},
        "gram_schmidt": {"one_projection_ms_per_solve": ms_step,
                         "reorthogonalized_ms_per_solve": float(np.mean(cgs2["ms"])),
                         "reorthogonalized_gmres_its": int(cgs2["out"]["gmres_its"][0]),
                         "reorthogonalized_newton_its": int(cgs2["out"]["newton_its"][0]),
                         "note": "GMRES orthogonalization: classical Gram-Schmidt with one projection (the "
                                 "headline) against one reorthogonalization"},
        "small_level_fusion": {"separate_ms_per_solve": ms_step, "fused_ms_per_solve": float(np.mean(fused["ms"])),
                               "cluster_tail_ms_per_solve": float(np.mean(tail["ms"])),
                               "cluster_tail_gmres_its": int(tail["out"]["gmres_its"][0]),
                               "note": "coarse levels as one launch per sweep, residual and transfer (the headline) "
                                       "against one cooperative launch per V-cycle for the levels below 20,000 "
                                       "nodes (fused) and one thread-block cluster launch for the levels of at "
                                       "most 160 nodes and the dense solve (cluster_tail)"},
        "autotune": None if tuned is None else {
            "config": tuned["config"], "ms_best_trial": tuned["ms"], "tuning_s": tuned["tuning_s"],
            "trials": [{"config": t["config"], "ms": t["ms"]} for t in tuned["trials"]],
            "learned_start": None if tuned_l is None else {"config": tuned_l["config"], "ms_best_trial": tuned_l["ms"],
                                                           "tuning_s": tuned_l["tuning_s"]}},
        "mixed_bphase_start": {"solves_per_s": 1000.0 / float(np.mean(ref_b["ms"])),
                               "newton_its": int(ref_b["out"]["newton_its"][0]),
                               "gmres_its": int(ref_b["out"]["gmres_its"][0]), "solver_config": cfg_b,
                               "start": "B phase + 0.05 N(0,1), seed 2"},
        "mixed_learned_start": None if alt is None else {
            "solves_per_s": 1000.0 / float(np.mean(alt["ms"])), "newton_its": int(alt["out"]["newton_its"][0]),
            "gmres_its": int(alt["out"]["gmres_its"][0]), "free_energy": alt["F"],
            "final_residual": float(alt["out"]["residual"][0]), "solver_config": cfg_l},
        "start": "learned (surrogate) guess" if use_learned else "B phase + 0.05 N(0,1)",
        "learned": learn_info,
        "mixed_vs_fp64": (1000.0 / ms_step) / (1000.0 / float(np.mean(fp64["ms"]))),
        "free_energy_rel_diff_vs_fp64": abs(mixed["F"] - fp64["F"]) / abs(fp64["F"]),
        "assembly_gdofs_mixed": nd / mixed["asm_ms"] / 1e6,
        "phases_ms": mixed["phases"],
        "kernel_ms": mixed["kernel_ms"],
        "kernel_launches": mixed["kernel_n"],
        "gpu_launches": int(mixed["launches"]),
        "roofline": {"bound": "hbm", "kernel": "k_mf_cell + k_mf_gather (matrix-free FP32 J z)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": MF_NCU_TRAFFIC,
                     "traffic_source": "dram read+write of one apply (both kernels) on the 32^3 cube, one ncu "
                                       "capture (dram__bytes_read.sum + dram__bytes_write.sum)",
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in pk else "fallback",
                     "algorithmic_bytes_per_launch": mf_bytes, "avg_launch_ms": mf_ms,
                     "fp32": {"achieved_tflops": mf_tflops, "peak_tflops": fp32_peak,
                              "frac": (mf_tflops / fp32_peak) if mf_tflops else None,
                              "flop_per_apply": mf_flop,
                              "peak_source": f"nominal CUDA-core FP32 ({n_sm} SMs x 128 lanes x 2) at the sampled SM clock",
                              "note": "the operator is bound by FP32 issue and latency, not HBM"},
                     "fp64_block_spmv": {"kernel": "k_spmv18<double>", "achieved": spmv_gbs,
                                         "frac": (spmv_gbs / hbm) if spmv_gbs else None,
                                         "algorithmic_bytes_per_launch": spmv_bytes, "avg_launch_ms": spmv_ms},
                     "assembly_algorithmic_bytes": asm_bytes},
        "e2e": {"value": e2e_val, "unit": "solves/s", "h2d_bytes_per_step": nd * 8, "d2h_bytes_per_step": nd * 8},
        "clocks": clk.summary(),
        "batched": batched,
    }
    try:
        sysr, x_or, line["cpu_baseline"] = cpu_port_baseline(args.linear_tol)
        line["err_vs_oracle"] = err_vs_oracle(sysr, x_or, mixed["x"], mixed["F"])
    except Exception as e:  # the CPU baseline must not hide the GPU line
        line["cpu_baseline"] = {"value": None, "error": str(e)}
    print(json.dumps(line))


def config3_leg(gl, linear_tol):
    """Mixed-precision solve of the refined cube: 64^3 Q1 on the same L = 20 cube, cells
    within 0.1 L of a z face refined once (hanging nodes on two interface planes), with
    multigrid (first coarse level: the unrefined 64^3 grid) and with block-Jacobi, against
    the FP64 GPU Newton on the same mesh and start (multigrid, and the plain block-Jacobi
    method)."""
    m = gl.cube_mesh(HALF, 64, 0.1)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=NOISE, seed=SEED)
    res = {"n_nodes": m.nn, "n_dofs": 18 * m.nn, "n_hanging": m.n_hanging, "n_cells": m.nc}
    legs = (("mixed", gl.MIXED, gl.PC_MULTIGRID), ("mixed_bj", gl.MIXED, gl.PC_BLOCK_JACOBI),
            ("fp64_mg", gl.FP64, gl.PC_MULTIGRID), ("fp64", gl.FP64, gl.PC_BLOCK_JACOBI))
    for name, prec, pc in legs:
        f = gl.FemGL(m, gl.Params.from_matep(P_BAR, T_RED, precision=prec, precond=pc))
        f.set_solution(x0)
        f.sync()
        f.event_start()
        o = f.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL, allow_unconverged=True)
        ms = f.event_stop()
        F = float(f.free_energy()[0])
        res[name] = {"ms": ms, "newton_its": int(o["newton_its"][0]), "gmres_its": int(o["gmres_its"][0]),
                     "final_residual": float(o["residual"][0]), "converged": bool(o["converged"]), "F": F,
                     "mg_levels": f.mg_levels, "mg_fallbacks": f.mg_fallbacks, "phases_ms": f.timers()}
        f.close()
    res["free_energy_rel_diff"] = abs(res["mixed"]["F"] - res["fp64"]["F"]) / abs(res["fp64"]["F"])
    res["mixed_vs_fp64"] = res["fp64"]["ms"] / res["mixed"]["ms"]
    res["mixed_vs_fp64_mg"] = res["fp64_mg"]["ms"] / res["mixed"]["ms"]
    return res


def config4_leg(gl, count, linear_tol):
    """The batched sweep at full scale: `count` seeded slab instances of the phase-diagram
    sweep (T/Tc ~ U(0.3, 0.95), p ~ U(0, 34) bar, D ~ U(8, 40) xi0, n ~ U{16..48} cells per
    side), mixed precision with multigrid, solved in waves of batched contexts that fit the
    device.  FP64 multigrid solves of the first instances, one at a time, check the free
    energies."""
    S = importlib.import_module("verkko-hem-repo_gb300.sweep")
    t0 = time.perf_counter()
    inst = batch_instances(gl, count)
    mesh_s = time.perf_counter() - t0
    meshes = [d["mesh"] for d in inst]
    prms = [gl.Params.from_matep(d["p"], d["t"], precision=gl.MIXED, precond=gl.PC_MULTIGRID) for d in inst]
    x0 = [d["x0"] for d in inst]
    S.solve_sweep(gl, meshes[:2], prms[:2], x0[:2], linear_tol=linear_tol, converge_acc=TOL)  # warm-up
    t0 = time.perf_counter()
    r = S.solve_sweep(gl, meshes, prms, x0, linear_tol=linear_tol, converge_acc=TOL,
                      log=lambda s: print(s, file=sys.stderr, flush=True))
    wall_s = time.perf_counter() - t0
    solve_s = sum(r["solve_ms"]) / 1000.0
    # FP64 GPU Newton one instance at a time, on a sample stratified by size (every
    # (count/8)-th instance in size order): with the same multigrid preconditioner, and the
    # plain method (block-Jacobi GMRES); the sample's mean time per solve scales to the sweep
    order = np.argsort([m.nn for m in meshes], kind="stable")
    sample = [int(order[k]) for k in range(0, count, max(1, count // 8))][:8]
    rel, t_mg, t_plain = [], [], []
    for i in sample:
        d = inst[i]
        for pc, acc in ((gl.PC_MULTIGRID, t_mg), (gl.PC_BLOCK_JACOBI, t_plain)):
            prm = gl.Params.from_matep(d["p"], d["t"], precision=gl.FP64, precond=pc)
            with gl.FemGL(d["mesh"], prm) as g:
                g.set_solution(d["x0"])
                g.sync()
                g.event_start()
                g.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL)
                acc.append(g.event_stop() / 1000.0)
                if pc == gl.PC_MULTIGRID:
                    Fd = g.free_energy()[0]
                    rel.append(abs(r["free_energy"][i] - Fd) / abs(Fd))
    fp64_mg_est = count * float(np.mean(t_mg))
    plain_est = count * float(np.mean(t_plain))
    return {"instances": count, "total_nodes": int(sum(m.nn for m in meshes)),
            "fp64_multigrid_one_at_a_time_solves_per_s_est": count / fp64_mg_est,
            "plain_fp64_one_at_a_time_solves_per_s_est": count / plain_est,
            "speedup_vs_fp64_multigrid_est": fp64_mg_est / solve_s,
            "speedup_vs_plain_fp64_est": plain_est / solve_s,
            "fp64_sample": {"instances": sample, "nodes": [int(meshes[i].nn) for i in sample],
                            "fp64_multigrid_s": t_mg, "plain_fp64_s": t_plain,
                            "note": "FP64 GPU Newton one instance at a time on 8 instances stratified by size; "
                                    "the sweep's FP64 time is count x the sample's mean"},
            "total_dofs": int(sum(18 * m.nn for m in meshes)),
            "solves_per_s": count / solve_s, "solves_per_s_with_setup": count / wall_s,
            "solve_s": solve_s, "setup_s": float(sum(r["create_s"])), "wall_s": wall_s, "mesh_s": mesh_s,
            "waves": r["waves"], "solve_ms_per_wave": r["solve_ms"], "create_s_per_wave": r["create_s"],
            "wave_gib": [b / 2**30 for b in r["wave_bytes"]], "bytes_per_node": r["bytes_per_node"],
            "budget_gib": r["budget"] / 2**30, "mg_fallbacks": r["mg_fallbacks"],
            "handed_off": [int(i) for i in np.flatnonzero(r["handed_off"])], "handoff_ms_per_wave": r["handoff_ms"],
            "handoff_note": "instances whose mixed multigrid solve stalled twice leave their wave at the state they "
                            "reached and are finished alone (two pre- and post-sweeps, then FP64); their device time "
                            "is part of solve_ms_per_wave",
            "all_converged": bool(r["converged"].all()), "max_final_residual": float(r["residual"].max()),
            "newton_its_mean": float(r["newton_its"].mean()), "gmres_its_mean": float(r["gmres_its"].mean()),
            "free_energy_rel_diff_vs_fp64_sample": rel,
            "sample": "seeded (seed 4) instances of the sweep: T/Tc~U(0.3,0.95), p~U(0,34), D~U(8,40), n~U{16..48}"}


def config5_leg(gl, n_train, n_test, linear_tol, n_test_cells=48):
    """The learned initial guess at scale: the surrogate is trained on n_train converged
    slab states (seeded (t, p, D), 8^3-12^3 cells, solved in waves from the uniform B
    phase), then n_test held-out (t, p, D) slab instances of n_test_cells^3 cells are
    solved in waves (mixed precision, multigrid) from three starts on the same wave
    contexts: the surrogate's guess (its inference inside the timed region), the
    configurations' B phase + 0.05 N(0,1), and the uniform B phase.  Reports solves/s,
    Newton and GMRES iterations and the free-energy agreement between the starts."""
    L = importlib.import_module("verkko-hem-repo_gb300.learned")
    S = importlib.import_module("verkko-hem-repo_gb300.sweep")
    t0 = time.perf_counter()
    X, Y, ginfo = L.generate(gl, n_train, seed=11, n_lo=8, n_hi=12, per_instance=512, waves=True)
    t_gen = time.perf_counter() - t0
    sur, tinfo = L.train(gl, X, Y, steps=3000, batch=8192, lr=1e-3, seed=0)
    rng = np.random.default_rng(55)
    test = []
    for _ in range(n_test):
        t = float(rng.uniform(0.3, 0.95))
        p = float(min(rng.uniform(0.0, 34.0), 34.0 - 1e-9))
        D = float(rng.uniform(8.0, 40.0))
        test.append((t, p, D))

    def make(k):
        t, p, D = test[k]
        m = gl.box_mesh([-L.L_HALF, -L.L_HALF, -D / 2], [L.L_HALF, L.L_HALF, D / 2], (n_test_cells,) * 3)
        return L.Instance(t, p, D, n_test_cells, m)

    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        test = list(ex.map(make, range(n_test)))
    prms = [gl.Params.from_matep(d.p, d.t, precision=gl.MIXED, precond=gl.PC_MULTIGRID) for d in test]
    meshes = [d.mesh for d in test]
    slope, const = S.footprint(gl, meshes, prms)
    free, _ = gl.mem_info()
    waves = S.plan_waves([m.nn for m in meshes], slope * 1.1, 0.9 * free - 2.0 * 2**30, const * 1.1)
    starts = {
        "learned": lambda idx: L.guess(gl, sur, [test[i] for i in idx]),
        "bphase_noise": lambda idx: [gl.bphase_guess(test[i].p, test[i].t, test[i].mesh.nn, noise=NOISE, seed=7000 + i)
                                     for i in idx],
        "bphase_uniform": lambda idx: [gl.bphase_guess(test[i].p, test[i].t, test[i].mesh.nn) for i in idx],
    }
    acc = {k: {"s": 0.0, "start_s": 0.0, "newton": [], "gmres": [], "res": [], "F": [], "ok": []} for k in starts}
    setup_s = 0.0
    for w in waves:
        t0 = time.perf_counter()
        with gl.FemGL([meshes[i] for i in w], [prms[i] for i in w]) as f:
            setup_s += time.perf_counter() - t0
            # untimed warm-up: one-time work of a new context (V-cycle graph capture, kernel
            # attributes) is paid before any start is timed
            f.set_solution(np.concatenate(starts["bphase_uniform"](w)))
            f.assemble_system()
            f.solve(1e-1, allow_unconverged=True)
            for name, mk in starts.items():
                t0 = time.perf_counter()
                x0 = np.concatenate(mk(w))  # inference (learned start) is timed with the solve
                f.set_solution(x0)
                f.sync()
                t_start = time.perf_counter() - t0
                f.event_start()
                o = f.run(max_newton=40, linear_tol=linear_tol, converge_acc=TOL, allow_unconverged=True)
                a = acc[name]
                a["s"] += f.event_stop() / 1000.0 + t_start
                a["start_s"] += t_start
                a["newton"] += o["newton_its"].tolist()
                a["gmres"] += o["gmres_its"].tolist()
                a["res"] += o["residual"].tolist()
                a["F"] += f.free_energy().tolist()
    sur.close()
    out = {"train": {"states": ginfo["converged"], "instances": n_train, "rows": tinfo["rows"],
                     "generation_s": t_gen, "training_s": tinfo["train_s"], "loss": tinfo["loss"],
                     "components_kept": tinfo["components_kept"]},
           "test_instances": n_test, "test_cells": n_test_cells, "waves": [len(w) for w in waves],
           "context_setup_s": setup_s}
    F = {k: np.array(a["F"]) for k, a in acc.items()}
    for name, a in acc.items():
        out[name] = {"solves_per_s": n_test / a["s"], "time_s": a["s"], "start_s": a["start_s"],
                     "solves_per_s_solve_only": n_test / (a["s"] - a["start_s"]),
                     "newton_its_total": int(sum(a["newton"])), "gmres_its_total": int(sum(a["gmres"])),
                     "newton_its_mean": float(np.mean(a["newton"])), "gmres_its_mean": float(np.mean(a["gmres"])),
                     "all_converged": bool(np.all(np.array(a["res"]) <= TOL)), "max_final_residual": float(max(a["res"]))}
    for name in ("bphase_noise", "bphase_uniform"):
        rel = np.abs(F["learned"] - F[name]) / np.abs(F[name])
        out[f"learned_speedup_vs_{name}"] = out["learned"]["solves_per_s"] / out[name]["solves_per_s"]
        out[f"max_free_energy_rel_diff_vs_{name}"] = float(rel.max())
        # instances whose two starts ended at different stationary points, and which start
        # found the lower free energy there
        diff = rel > 1e-9
        out[f"instances_other_stationary_point_vs_{name}"] = int(diff.sum())
        out[f"of_those_learned_lower_F_vs_{name}"] = int(np.sum(diff & (F["learned"] < F[name])))
        out[f"median_free_energy_rel_diff_vs_{name}"] = float(np.median(rel))
    return out


def ncu_case(n, fp64):
    """Small fixed workload for ncu captures (committed so profiles name runnable commands)."""
    gl = importlib.import_module("verkko-hem-repo_gb300")
    gl.build()
    m = gl.cube_mesh(HALF, n)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=NOISE, seed=SEED)
    prm = gl.Params.from_matep(P_BAR, T_RED, precision=gl.FP64 if fp64 else gl.MIXED, gmres_max_iter=30)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        rn = f.assemble_system()
        its = f.solve(1e-12, allow_unconverged=True)
        f.sync()
        print(json.dumps({"ncu_case": n, "fp64": bool(fp64), "rhs_norm": float(rn[0]), "gmres_its": int(its[0]),
                          "launches": f.launch_count}))
    return 0


def ncu_solve(n, fp64, precond, prec_reuse=0.0):
    """One complete Newton solve of the workload's physics on an n^3 cube (profiling case)."""
    gl = importlib.import_module("verkko-hem-repo_gb300")
    gl.build()
    m = gl.cube_mesh(HALF, n)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=NOISE, seed=SEED)
    pc = gl.PC_MULTIGRID if precond == "mg" else gl.PC_BLOCK_JACOBI
    prm = gl.Params.from_matep(P_BAR, T_RED, precision=gl.FP64 if fp64 else gl.MIXED, precond=pc,
                               prec_reuse=prec_reuse)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        out = f.run(max_newton=40, linear_tol=1e-4, converge_acc=TOL)
        print(json.dumps({"ncu_solve": n, "fp64": bool(fp64), "precond": precond, "prec_reuse": prec_reuse,
                          "newton_its": int(out["newton_its"][0]), "gmres_its": int(out["gmres_its"][0]),
                          "residual": float(out["residual"][0]), "launches": f.launch_count}))
    return 0


def reference_arm(args, rank):
    """The reference's CPU implementation of the path, timed on this host's cores.

    The reference program needs deal.II/Trilinos/p4est/MPI, none of which exist here, so
    each step is one complete FP64 Newton solve of the workload by the oracle port (the
    reference's algorithm restated in C with OpenMP on all host cores, block-Jacobi
    GMRES in place of ML AMG), built from oracle code alone: this process never loads
    the CUDA library.  Steps are a bounded sample: solves repeat until about two
    minutes have passed.  Where the reference's own kernels were compiled (only where
    the reference tree exists), their cell loop is timed beside it and extrapolated."""
    if rank != 0:
        return 0
    sysr, x0 = oracle_problem()
    for _ in range(args.warmup):  # warm-up: assemblies of the object that is timed
        sysr.assemble(sysr.distribute(x0), want_J=False)
    dt, ns, nn, gi, thr, res = cpu_solves(sysr, x0, args.linear_tol, budget_s=120.0)
    value = 1.0 / dt
    kern = reference_kernels_leg(sysr, x0, thr)
    with open("/proc/self/maps") as fh:
        if "libglgpu" in fh.read():
            raise RuntimeError("the reference arm loaded the CUDA library")
    sample = (f"{ns} complete FP64 Newton solve(s) on {thr} host threads with the oracle port "
              f"({nn} Newton its, {gi} block-Jacobi GMRES(50) its, final |F| {res:.2e}, {dt:.1f} s per solve)")
    print(json.dumps({"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": 1000.0 * dt, "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded B-phase + Gaussian noise start)",
                      "config": bench_config(args.linear_tol), "impl": "reference",
                      "solver": {"method": "FP64 Newton, block-Jacobi GMRES(50), the reference's line search",
                                 "solves_timed": ns, "newton_its": nn, "gmres_its": gi, "final_residual": res},
                      "cpu_baseline": {"value": value, "unit": "solves/s", "cores": thr, "kind": "port",
                                       "sample": sample},
                      "reference_kernels": kern,
                      "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


if __name__ == "__main__":
    sys.exit(main() or 0)
