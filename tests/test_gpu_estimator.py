"""GPU Kelly error estimator and fixed-number refinement flags against the oracle's
restatement (oracle/kelly.py: neighbours by point location, not by the product's node keys),
and one adaptive cycle (estimate, flag, refine, transfer, solve) as the reference's
refine_grid("adaptive") does it (femgl/src/refine.cc:131-176).

Tolerances: the estimate is returned in FP32 (deal.II's Vector<float>), so 2e-6 relative to
the largest value; flags are compared exactly given the same estimates."""
import numpy as np
import pytest

from _lib import coef_of, oracle_mesh, product

pytestmark = pytest.mark.gpu

P_BAR, T_RED = 20.0, 0.6
LO, HI, N = [-2.0, -2.5, -1.5], [2.0, 2.5, 1.5], (4, 5, 3)


@pytest.fixture(scope="module")
def gl():
    return product()


def _mesh(gl, kind):
    if kind == "uniform":
        return gl.box_mesh(LO, HI, N), (0, 0)
    if kind == "band":
        return gl.box_mesh(LO, HI, N, refine_band=0.9), (0, 0)
    if kind == "periodic":
        return gl.box_mesh(LO, HI, N, periodic_xy=(1, 1)), (1, 1)
    if kind == "periodic_band":
        return gl.box_mesh(LO, HI, N, refine_band=0.9, periodic_xy=(1, 1)), (1, 1)
    flags = np.zeros(np.prod(N), np.int8)
    flags[np.random.default_rng(8).choice(flags.size, 17, replace=False)] = 1
    return gl.box_mesh_refine(LO, HI, N, flags), (0, 0)


@pytest.mark.parametrize("kind", ["uniform", "band", "periodic", "periodic_band", "flags"])
def test_kelly_matches_oracle(gl, oracle_gl, kind):
    from oracle import kelly as ok

    m, per = _mesh(gl, kind)
    prm = gl.Params.from_matep(P_BAR, T_RED)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.4, seed=11)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr = sysr.distribute(x0)
    ref = ok.kelly(oracle_mesh(m), xr, LO, HI, N, periodic=per)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        eta = f.estimate_error()
    assert eta.dtype == np.float32 and eta.shape == (m.nc,)
    assert np.abs(eta - ref).max() <= 2e-6 * ref.max()


def test_refine_flags_per_instance(gl):
    from oracle import kelly as ok

    m1, _ = _mesh(gl, "band")
    m2 = gl.cube_mesh(3.0, 5)
    x = np.concatenate([gl.bphase_guess(P_BAR, T_RED, m1.nn, noise=0.3, seed=1),
                        gl.bphase_guess(P_BAR, T_RED, m2.nn, noise=0.3, seed=2)])
    prm = gl.Params.from_matep(P_BAR, T_RED)
    with gl.FemGL([m1, m2], [prm, prm]) as f:
        f.set_solution(x)
        with pytest.raises(gl.GLGPUError):
            f.refine_flags(0.3)  # no estimate yet
        eta = f.estimate_error()
        for top, bottom in ((0.3, 0.0), (0.3, 0.1), (0.0, 0.25), (1.0, 0.0)):
            flags = f.refine_flags(top, bottom)
            for sl in (slice(0, m1.nc), slice(m1.nc, m1.nc + m2.nc)):
                assert np.array_equal(flags[sl], ok.fixed_number_flags(eta[sl], top, bottom))
        assert (f.refine_flags(0.3)[: m1.nc] == 1).sum() == int(0.3 * m1.nc)


def test_adaptive_cycle(gl, oracle_gl):
    """Solve, estimate, refine the top 30 %, transfer the solution, solve again; the refined
    solve follows the oracle's Newton path from the transferred state."""
    lo, hi, n = [-4.0, -4.0, -4.0], [4.0, 4.0, 4.0], (6, 6, 6)
    m = gl.box_mesh(lo, hi, n)
    prm = gl.Params.from_matep(P_BAR, T_RED, precision=gl.MIXED, precond=gl.PC_MULTIGRID)
    with gl.FemGL(m, prm) as f:
        f.set_solution(gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.05, seed=2))
        out = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        assert out["converged"]
        xc = f.solution()
        f.estimate_error()
        flags = f.refine_flags(0.3)
    assert flags.sum() >= int(0.3 * m.nc)
    mf = gl.box_mesh_refine(lo, hi, n, flags)
    assert mf.nc == m.nc + 7 * int(flags.sum()) and mf.n_hanging > 0
    x1 = gl.box_interpolate(lo, hi, n, xc, mf.xyz)
    prm_f = gl.Params.from_matep(P_BAR, T_RED)
    sysr = oracle_gl.System(oracle_mesh(mf), coef_of(prm_f))
    xr, hist = oracle_gl.newton(sysr, x1, tol=1e-10, max_iter=40)
    _, Fr = sysr.residual(xr)
    with gl.FemGL(mf, prm_f) as f:
        f.set_solution(x1)
        assert np.allclose(f.solution(), sysr.distribute(x1), rtol=0, atol=1e-15)
        out = f.run(max_newton=40, linear_tol=1e-12, converge_acc=1e-10)
        F = f.free_energy()
    assert out["converged"] and out["residual"][0] <= 1e-10
    assert out["newton_its"][0] == len(hist)
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)
