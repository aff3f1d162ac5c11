"""Geometric multigrid preconditioner (flexible GMRES) on the GPU: tight linear solves
agree with the oracle's Jacobian, Newton with multigrid reproduces the oracle's answer,
batched instances of different sizes work, and non-uniform (refined) meshes fall back
to block-Jacobi."""
import numpy as np
import pytest

from _lib import coef_of, oracle_mesh, product

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gl():
    return product()


def _solve(gl, m, x0, precond, precision=0, tol=1e-10):
    prm = gl.Params.from_matep(20.0, 0.6, precond=precond, precision=precision)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        its = f.solve(tol)
        d = f.update()
        _, _, J, rhs = f.system()
        lev = f.mg_levels
    return its[0], d, J, rhs, lev


@pytest.mark.parametrize("n", [8, 7])
def test_multigrid_tight_solve(gl, oracle_gl, n):
    m = gl.cube_mesh(5.0, n)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=3)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(gl.Params.from_matep(20.0, 0.6)))
    its_mg, d, J, rhs, lev = _solve(gl, m, x0, gl.PC_MULTIGRID)
    its_bj, _, _, _, _ = _solve(gl, m, x0, gl.PC_BLOCK_JACOBI)
    assert lev >= 3
    r = sysr.spmv(J, d) - rhs
    r[~sysr.free] = 0.0
    assert np.linalg.norm(r) <= 2e-10 * np.linalg.norm(rhs)
    assert its_mg < its_bj, (its_mg, its_bj)


def test_newton_multigrid_matches_oracle(gl, oracle_gl):
    m = gl.cube_mesh(2.5, 4)
    prm = gl.Params.from_matep(20.0, 0.6, precond=gl.PC_MULTIGRID)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=2)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr, hist = oracle_gl.newton(sysr, x0, tol=1e-10, max_iter=40)
    _, Fr = sysr.residual(xr)
    for precision in (gl.FP64, gl.MIXED):
        prm.precision = precision
        with gl.FemGL(m, prm) as f:
            f.set_solution(x0)
            out = f.run(max_newton=40, linear_tol=1e-12 if precision == gl.FP64 else 1e-4, converge_acc=1e-10)
            x, F = f.solution(), f.free_energy()
        assert out["converged"]
        if precision == gl.FP64:
            assert out["newton_its"][0] == len(hist)
            assert np.abs(x - xr).max() <= 1e-9 * np.abs(xr).max()
        assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)


def test_multigrid_batched_uneven(gl):
    meshes = [gl.box_mesh([-10, -10, -4], [10, 10, 4], (9, 9, 9)), gl.cube_mesh(5.0, 6),
              gl.box_mesh([-10, -10, -12], [10, 10, 12], (12, 12, 12))]
    pts = [(20.0, 0.6), (12.0, 0.45), (30.0, 0.85)]
    x0 = np.concatenate([gl.bphase_guess(p, t, m.nn, noise=0.05, seed=k) for k, (m, (p, t)) in
                         enumerate(zip(meshes, pts))])
    res = {}
    for pc in (gl.PC_BLOCK_JACOBI, gl.PC_MULTIGRID):
        prms = [gl.Params.from_matep(p, t, precond=pc, precision=gl.MIXED) for p, t in pts]
        with gl.FemGL(meshes, prms) as f:
            f.set_solution(x0)
            out = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
            res[pc] = (out, f.free_energy(), f.mg_levels)
    ob, Fb, _ = res[gl.PC_BLOCK_JACOBI]
    om, Fm, lev = res[gl.PC_MULTIGRID]
    assert lev >= 3 and om["converged"] and ob["converged"]
    assert np.allclose(Fm, Fb, rtol=1e-9)
    assert om["gmres_its"].sum() < ob["gmres_its"].sum()


def test_multigrid_falls_back_on_refined_mesh(gl):
    m = gl.cube_mesh(2.5, 4, 0.25)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=1)
    its, d, J, rhs, lev = _solve(gl, m, x0, gl.PC_MULTIGRID)
    assert lev == 0 and its > 0
