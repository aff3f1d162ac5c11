"""GPU parity at the benchmark configurations' full sizes, against the FP64 CPU oracle.

* femgl 3D, 32^3 Q1 cube (L = 20, p = 20 bar, t = 0.6, z-face pair breaking, B phase
  + 0.05 N(0,1), seed 2; 646,866 unknowns): the FP64 Jacobian on the unconstrained
  block and the residual to 1e-12 relative, the free energy to 1e-12; the FP64 Newton
  solve with the same linear tolerance on both sides (1e-6: near the solution the exact
  phase and spin-rotation symmetries make the Jacobian nearly singular, and the oracle's
  block-Jacobi GMRES stalls at tighter tolerances): equal Newton counts, the converged
  order parameter (up to the functional's exact global phase and spin-rotation
  symmetries) and free energy to 1e-9 relative; the mixed-precision multigrid solve (the
  benchmark's headline method): its FP64 stop-test residual re-evaluated by the oracle,
  and its order parameter and free energy against the oracle's converged solve to 1e-9.
* the refined 64^3 cube (cells within 0.1 L of the z faces refined once; hanging
  nodes; 11.7M unknowns): the mixed solve's state checked by the oracle's FP64
  residual and free energy, and against the FP64 GPU solve.

The reference loops these restate: femgl/src/assemble.cc:188-280 (assembly),
residual.cc:166-291, iteration.cc:128-210 (damped Newton), run.cc:234 (stop rule).
"""
import numpy as np
import pytest

from _lib import coef_of, oracle_mesh, product

pytestmark = pytest.mark.gpu

P_BAR, T_RED, HALF, NOISE, SEED = 20.0, 0.6, 10.0, 0.05, 2
LIN_TOL = 1e-6


@pytest.fixture(scope="module")
def gl():
    return product()


@pytest.fixture(scope="module")
def cube32(gl, oracle_gl):
    m = gl.cube_mesh(HALF, 32)
    prm = gl.Params.from_matep(P_BAR, T_RED)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=NOISE, seed=SEED)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    return m, x0, sysr


@pytest.fixture(scope="module")
def oracle_solution32(cube32, oracle_gl):
    """The oracle's converged FP64 Newton solve of the 32^3 workload, GMRES to 1e-6."""
    m, x0, sysr = cube32
    x, hist = oracle_gl.newton(sysr, x0, tol=1e-10, max_iter=40, linear_tol=LIN_TOL)
    R, F = sysr.residual(x)
    return x, hist, F, float(np.linalg.norm(R))


def _free_block_err_chunked(sysr, J_gpu, J_ref, chunk=65536):
    free = sysr.free.reshape(-1, 18)
    rows = np.repeat(np.arange(sysr.m.nn), np.diff(sysr.rowptr))
    num = den = 0.0
    for a in range(0, sysr.nnzb, chunk):
        b = min(a + chunk, sysr.nnzb)
        mask = free[rows[a:b]][:, :, None] & free[sysr.cols[a:b]][:, None, :]
        num = max(num, float(np.abs(np.where(mask, J_gpu[a:b] - J_ref[a:b], 0.0)).max()))
        den = max(den, float(np.abs(np.where(mask, J_ref[a:b], 0.0)).max()))
    return num / den


def test_config2_fp64_assembly_full_size(gl, cube32):
    m, x0, sysr = cube32
    xr = sysr.distribute(x0)
    Jr, Rr, Fr = sysr.assemble(xr)
    prm = gl.Params.from_matep(P_BAR, T_RED, precision=gl.FP64)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        rn = f.assemble_system()
        rowptr, cols, J, rhs = f.system()
        F = f.free_energy()
    assert J.shape[0] == 912673 and 18 * m.nn == 646866
    assert np.array_equal(rowptr, sysr.rowptr) and np.array_equal(cols, sysr.cols)
    assert _free_block_err_chunked(sysr, J, Jr) <= 1e-12
    assert np.abs(rhs + Rr).max() <= 1e-12 * np.abs(Rr).max()
    assert abs(rn[0] - np.linalg.norm(Rr)) <= 1e-12 * np.linalg.norm(Rr)
    assert abs(F[0] - Fr) <= 1e-12 * abs(Fr)


def test_config2_fp64_newton_matches_oracle(gl, oracle_gl, cube32, oracle_solution32):
    m, x0, sysr = cube32
    xr, hist, Fr, nr = oracle_solution32
    assert nr <= 1e-10
    prm = gl.Params.from_matep(P_BAR, T_RED, precision=gl.FP64, precond=gl.PC_MULTIGRID)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        out = f.run(max_newton=40, linear_tol=LIN_TOL, converge_acc=1e-10)
        x = f.solution()
        F = f.free_energy()
    assert out["converged"] and out["residual"][0] <= 1e-10
    assert out["newton_its"][0] == len(hist), (out["newton_its"], [h["res"] for h in hist])
    # the order parameter up to the functional's exact symmetries (global phase, spin
    # rotation): the Jacobian is singular along them, so the two Newton runs, whose linear
    # solves differ, stop at different points of the same orbit (2e-7 apart here)
    xa, _, _ = oracle_gl.gauge_align(x, xr)
    assert np.abs(xa - xr).max() <= 1e-9 * np.abs(xr).max(), np.abs(xa - xr).max()
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)
    # the GPU's converged state, checked by the oracle's own residual
    Rg, Fg = sysr.residual(x)
    assert np.linalg.norm(Rg) <= 1.5e-10
    assert abs(Fg - F[0]) <= 1e-12 * abs(Fg)


def test_config2_mixed_multigrid_matches_oracle(gl, oracle_gl, cube32, oracle_solution32):
    """The headline method: FP32 Jacobian and flexible GMRES with multigrid, FP64
    stop test; the answer is the FP64 oracle's."""
    m, x0, sysr = cube32
    xr, hist, Fr, _ = oracle_solution32
    prm = gl.Params.from_matep(P_BAR, T_RED, precision=gl.MIXED, precond=gl.PC_MULTIGRID)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        out = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        x = f.solution()
        F = f.free_energy()
    assert out["converged"]
    assert out["residual"][0] == out["residual_fp64"][0] <= 1e-10
    Rg, Fg = sysr.residual(x)
    # the FP64 stop-test value is the oracle's residual norm at the same state.  At a
    # converged state |R| ~ 1e-11 is what is left of O(1) terms that cancel, so two FP64
    # evaluations that sum in different orders agree on it to ~1e-15 absolute (1e-5 relative)
    assert abs(np.linalg.norm(Rg) - out["residual_fp64"][0]) <= 1e-14, (np.linalg.norm(Rg), out["residual_fp64"])
    assert np.linalg.norm(Rg) <= 1.5e-10
    assert abs(F[0] - Fg) <= 1e-12 * abs(Fg)
    # up to the exact symmetries (see the FP64 test)
    xa, _, _ = oracle_gl.gauge_align(x, xr)
    assert np.abs(xa - xr).max() <= 1e-9 * np.abs(xr).max(), np.abs(xa - xr).max()
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)


def test_config3_refined_mixed_error_vs_oracle(gl, oracle_gl):
    """Config 3: 64^3 with a refined band at the z faces (hanging nodes).  The mixed
    multigrid solve's state is checked by the oracle's FP64 residual and free energy,
    and its free energy against the FP64 GPU solve of the same mesh and start."""
    m = gl.cube_mesh(HALF, 64, 0.1)
    assert m.n_hanging > 0 and 18 * m.nn > 10_000_000
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=NOISE, seed=SEED)
    prm_m = gl.Params.from_matep(P_BAR, T_RED, precision=gl.MIXED, precond=gl.PC_MULTIGRID)
    with gl.FemGL(m, prm_m) as f:
        f.set_solution(x0)
        out = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        x = f.solution()
        F = f.free_energy()[0]
    assert out["converged"] and out["residual_fp64"][0] <= 1e-10
    prm_d = gl.Params.from_matep(P_BAR, T_RED, precision=gl.FP64, precond=gl.PC_MULTIGRID)
    with gl.FemGL(m, prm_d) as f:
        f.set_solution(x0)
        out_d = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        x_d = f.solution()
        F_d = f.free_energy()[0]
    assert out_d["converged"]
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm_m))
    Rg, Fg = sysr.residual(x)
    assert np.linalg.norm(Rg) <= 1.5e-10
    assert abs(F - Fg) <= 1e-12 * abs(Fg)
    assert abs(F - F_d) <= 1e-9 * abs(F_d)
    xa, _, _ = oracle_gl.gauge_align(x, x_d)
    assert np.abs(xa - x_d).max() <= 1e-9 * np.abs(x_d).max(), np.abs(xa - x_d).max()
