"""Robin (AdGR) faces on the GPU against the FP64 oracle: with the diffuse length bt < 1e10
the pair-breaking faces add (K1/bt) int |A_t|^2 dS (femgl/src/assemble.cc:286-348,
residual.cc:235-278).  The oracle's face term is pinned to the reference's own face loop by
tests/golden/face.npz.

Tolerances as in the bulk parity tests: FP64 Jacobian, residual and energy 1e-12 relative;
FP32 (mixed) operator 2e-5 of the row scale; free energies of converged states 1e-9, the
states themselves 1e-6 (soft directions of the B phase)."""
import numpy as np
import pytest

from _lib import coef_of, oracle_mesh, product

pytestmark = pytest.mark.gpu

P_BAR, T_RED = 20.0, 0.6
BT = 1.5


@pytest.fixture(scope="module")
def gl():
    return product()


def _free_block_err(sysr, J_gpu, J_ref):
    free = sysr.free.reshape(-1, 18)
    rows = np.repeat(np.arange(sysr.m.nn), np.diff(sysr.rowptr))
    mask = free[rows][:, :, None] & free[sysr.cols][:, None, :]
    d = np.where(mask, J_gpu - J_ref, 0.0)
    return np.abs(d).max() / np.abs(np.where(mask, J_ref, 0.0)).max()


def _mesh(gl, dxy=(1, 1), frac=0.25, n=(4, 5, 4)):
    return gl.box_mesh([-1.0, -1.5, -1.25], [1.0, 1.5, 1.25], n, refine_band=frac * 2.5, dirichlet_xy=dxy)


@pytest.mark.parametrize("dxy,frac", [((0, 0), 0.0), ((1, 1), 0.25), ((1, 0), 0.3)])
def test_robin_assembly_fp64_matches_oracle(gl, oracle_gl, dxy, frac):
    m = _mesh(gl, dxy, frac)
    prm = gl.Params.from_matep(P_BAR, T_RED, bt=BT)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.3, seed=5)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr = sysr.distribute(x0)
    Jr, Rr, Fr = sysr.assemble(xr)
    # the face term is really there: the same state without it differs
    sys0 = oracle_gl.System(oracle_mesh(m), coef_of(gl.Params.from_matep(P_BAR, T_RED)))
    _, R0, F0 = sys0.assemble(xr)
    assert np.abs(Rr - R0).max() > 1e-3 * np.abs(Rr).max() and abs(Fr - F0) > 1e-6 * abs(Fr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        rn = f.assemble_system()
        _, _, J, rhs = f.system()
        nr = f.compute_residual()
        R = f.residual()
        F = f.free_energy()
    assert _free_block_err(sysr, J, Jr) <= 1e-12
    assert np.abs(rhs + Rr).max() <= 1e-12 * np.abs(Rr).max()
    assert np.abs(R - Rr).max() <= 1e-12 * np.abs(Rr).max()
    assert abs(rn[0] - np.linalg.norm(Rr)) <= 1e-12 * np.linalg.norm(Rr)
    assert abs(nr[0] - np.linalg.norm(Rr)) <= 1e-12 * np.linalg.norm(Rr)
    assert abs(F[0] - Fr) <= 1e-12 * abs(Fr)


@pytest.mark.parametrize("frac", [0.25, 0.0])
def test_robin_mixed_matrix_free_operator(gl, oracle_gl, frac):
    m = _mesh(gl, (1, 1), frac)
    prm = gl.Params.from_matep(P_BAR, T_RED, bt=BT, precision=gl.MIXED)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.3, seed=6)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    Jr, Rr, _ = sysr.assemble(sysr.distribute(x0))
    v = np.random.default_rng(3).standard_normal(18 * m.nn)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        y = f.spmv(v)
        _, _, J, rhs = f.system()
    fr = sysr.free
    assert _free_block_err(sysr, J, Jr) <= 1e-5
    assert np.abs(rhs + Rr).max() <= 1e-12 * np.abs(Rr).max()
    v32 = v.astype(np.float32).astype(np.float64)
    y_ref = sysr.spmv(Jr, v32)
    scale = np.abs(y_ref[fr]).max()
    assert np.abs(y - sysr.spmv(J, v32))[fr].max() <= 2e-5 * scale
    assert np.abs(y - y_ref)[fr].max() <= 2e-5 * scale


def test_robin_newton_fp64_matches_oracle(gl, oracle_gl):
    # z faces pair-breaking with the Robin term; wide enough for a superfluid state
    m = gl.box_mesh([-4.0, -4.0, -4.0], [4.0, 4.0, 4.0], (4, 4, 4))
    prm = gl.Params.from_matep(P_BAR, T_RED, bt=BT)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.05, seed=2)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr, hist = oracle_gl.newton(sysr, x0, tol=1e-10, max_iter=40)
    _, Fr = sysr.residual(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        out = f.run(max_newton=40, linear_tol=1e-12, converge_acc=1e-10)
        x = f.solution()
        F = f.free_energy()
    assert out["converged"] and out["residual"][0] <= 1e-10
    assert np.abs(xr).max() > 0.5  # not the normal state
    assert out["newton_its"][0] == len(hist)
    # |R| < 1e-10 fixes the state only to |R| / (smallest Hessian eigenvalue): the B phase
    # keeps soft directions, and with these boundaries the GPU's and the oracle's Krylov
    # rounding leave the converged states ~1e-8 apart along them; the energy is quadratic
    # there and agrees to 1e-9
    assert np.abs(x - xr).max() <= 1e-6 * np.abs(xr).max()
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)


@pytest.mark.parametrize("precond", ["mg", "bj"])
def test_robin_newton_mixed_reaches_oracle_answer(gl, oracle_gl, precond):
    pc = gl.PC_MULTIGRID if precond == "mg" else gl.PC_BLOCK_JACOBI
    m = gl.box_mesh([-5.0, -5.0, -5.0], [5.0, 5.0, 5.0], (8, 8, 8), dirichlet_xy=(1, 1))
    prm = gl.Params.from_matep(P_BAR, T_RED, bt=BT, precision=gl.MIXED, precond=pc)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.05, seed=2)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr, _ = oracle_gl.newton(sysr, x0, tol=1e-10, max_iter=40)
    _, Fr = sysr.residual(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        out = f.run(max_newton=60, linear_tol=1e-4, converge_acc=1e-10)
        x = f.solution()
        F = f.free_energy()
        levels = f.mg_levels
    assert out["converged"] and out["residual"][0] <= 1e-10
    if precond == "mg":
        assert levels >= 1
    Rg, _ = sysr.residual(x)
    assert np.linalg.norm(Rg) <= 1.5e-10
    # the B phase keeps a continuous degeneracy, so the FP32 Krylov path may end at another
    # point of the same minimum: the energy is the comparable quantity
    assert np.abs(x).max() > 0.5
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)


def test_robin_batched_with_inactive_instance(gl, oracle_gl):
    """One context, two instances: Robin active in one, inactive (bt = 1e10) in the other."""
    m1 = gl.box_mesh([-2.5, -2.5, -2.5], [2.5, 2.5, 2.5], (4, 4, 4), dirichlet_xy=(1, 1))
    m2 = gl.cube_mesh(2.0, 4, 0.25)
    p1 = gl.Params.from_matep(P_BAR, T_RED, bt=BT)
    p2 = gl.Params.from_matep(10.0, 0.5)
    x1 = gl.bphase_guess(P_BAR, T_RED, m1.nn, noise=0.1, seed=1)
    x2 = gl.bphase_guess(10.0, 0.5, m2.nn, noise=0.1, seed=2)
    with gl.FemGL([m1, m2], [p1, p2]) as f:
        f.set_solution(np.concatenate([x1, x2]))
        f.compute_residual()
        R = f.residual()
        F = f.free_energy()
    for k, (m, p, x0) in enumerate(((m1, p1, x1), (m2, p2, x2))):
        sysr = oracle_gl.System(oracle_mesh(m), coef_of(p))
        _, Rr, Fr = sysr.assemble(sysr.distribute(x0), want_J=False)
        Rk = R[: 18 * m1.nn] if k == 0 else R[18 * m1.nn:]
        assert np.abs(Rk - Rr).max() <= 1e-12 * np.abs(Rr).max()
        assert abs(F[k] - Fr) <= 1e-12 * abs(Fr)
