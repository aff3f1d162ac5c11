"""Periodic x / y faces on the GPU against the FP64 oracle (the reference's
makegrid_retangle-z-AdGR_xy-periodic.cc scenario: z faces pair-breaking, optionally with the
AdGR Robin term, x / y periodic).  Periodicity enters as constraint rows of the same block
matrix; the oracle condenses them with its own independent code.

Tolerances as in the bulk parity tests: FP64 Jacobian, residual and energy 1e-12 relative;
FP32 (mixed) operator 2e-5 of the row scale; free energies of converged states 1e-9, the
states themselves 1e-6 (soft directions of the B phase)."""
import numpy as np
import pytest

from _lib import coef_of, oracle_mesh, product

pytestmark = pytest.mark.gpu

P_BAR, T_RED = 20.0, 0.6


@pytest.fixture(scope="module")
def gl():
    return product()


def _free_block_err(sysr, J_gpu, J_ref):
    free = sysr.free.reshape(-1, 18)
    rows = np.repeat(np.arange(sysr.m.nn), np.diff(sysr.rowptr))
    mask = free[rows][:, :, None] & free[sysr.cols][:, None, :]
    d = np.where(mask, J_gpu - J_ref, 0.0)
    return np.abs(d).max() / np.abs(np.where(mask, J_ref, 0.0)).max()


def _mesh(gl, per=(1, 1), frac=0.25, n=(4, 5, 4), half=(1.0, 1.5, 1.25)):
    lo = [-h for h in half]
    return gl.box_mesh(lo, list(half), n, refine_band=frac * 2 * half[2], periodic_xy=per)


@pytest.mark.parametrize("per,frac,bt", [((1, 1), 0.0, 1e10), ((1, 1), 0.25, 1.5), ((1, 0), 0.3, 1e10)])
def test_periodic_assembly_fp64_matches_oracle(gl, oracle_gl, per, frac, bt):
    m = _mesh(gl, per, frac)
    prm = gl.Params.from_matep(P_BAR, T_RED, bt=bt)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.3, seed=5)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr = sysr.distribute(x0)
    # the distributed state is periodic: every upper-face node equals its image
    lo, hi = m.xyz.min(0), m.xyz.max(0)
    index = {tuple(np.round(p, 9)): i for i, p in enumerate(m.xyz)}
    X = xr.reshape(-1, 18)
    for axis in range(2):
        if per[axis]:
            for i in np.nonzero(m.xyz[:, axis] == hi[axis])[0]:
                q = m.xyz[i].copy()
                q[axis] = lo[axis]
                assert np.array_equal(X[i], X[index[tuple(np.round(q, 9))]])
    Jr, Rr, Fr = sysr.assemble(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        x = f.solution()
        rn = f.assemble_system()
        _, _, J, rhs = f.system()
        nr = f.compute_residual()
        R = f.residual()
        F = f.free_energy()
        v = np.random.default_rng(2).standard_normal(18 * m.nn)
        y = f.spmv(v)
    assert np.allclose(x, xr, rtol=0, atol=1e-15)
    assert _free_block_err(sysr, J, Jr) <= 1e-12
    assert np.abs(rhs + Rr).max() <= 1e-12 * np.abs(Rr).max()
    assert np.abs(R - Rr).max() <= 1e-12 * np.abs(Rr).max()
    assert abs(rn[0] - np.linalg.norm(Rr)) <= 1e-12 * np.linalg.norm(Rr)
    assert abs(nr[0] - np.linalg.norm(Rr)) <= 1e-12 * np.linalg.norm(Rr)
    assert abs(F[0] - Fr) <= 1e-12 * abs(Fr)
    yr = sysr.spmv(Jr, v)
    fr = sysr.free
    assert np.abs(y - yr)[fr].max() <= 1e-12 * np.abs(yr[fr]).max()


@pytest.mark.parametrize("frac,bt", [(0.25, 1e10), (0.0, 1.5)])
def test_periodic_mixed_matrix_free_operator(gl, oracle_gl, frac, bt):
    m = _mesh(gl, (1, 1), frac)
    prm = gl.Params.from_matep(P_BAR, T_RED, bt=bt, precision=gl.MIXED)
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


@pytest.mark.parametrize("bt", [1e10, 3.0])
def test_periodic_newton_fp64_matches_oracle(gl, oracle_gl, bt):
    # a slab periodic in x and y between pair-breaking z walls
    m = gl.box_mesh([-4.0, -4.0, -4.0], [4.0, 4.0, 4.0], (4, 4, 4), periodic_xy=(1, 1))
    prm = gl.Params.from_matep(P_BAR, T_RED, bt=bt)
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
    assert np.abs(xr).max() > 0.5
    assert out["newton_its"][0] == len(hist)
    # |R| < 1e-10 fixes the state only to |R| / (smallest Hessian eigenvalue): the B phase
    # keeps soft directions, and with these boundaries the GPU's and the oracle's Krylov
    # rounding leave the converged states ~1e-8 apart along them; the energy is quadratic
    # there and agrees to 1e-9
    assert np.abs(x - xr).max() <= 1e-6 * np.abs(xr).max()
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)


@pytest.mark.parametrize("precond", ["mg", "bj"])
def test_periodic_newton_mixed_reaches_oracle_answer(gl, oracle_gl, precond):
    pc = gl.PC_MULTIGRID if precond == "mg" else gl.PC_BLOCK_JACOBI
    m = gl.box_mesh([-5.0, -5.0, -5.0], [5.0, 5.0, 5.0], (8, 8, 8), periodic_xy=(1, 1))
    prm = gl.Params.from_matep(P_BAR, T_RED, bt=3.0, precision=gl.MIXED, precond=pc)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.05, seed=2)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr, _ = oracle_gl.newton(sysr, x0, tol=1e-10, max_iter=40)
    _, Fr = sysr.residual(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        out = f.run(max_newton=60, linear_tol=1e-4, converge_acc=1e-10)
        x = f.solution()
        F = f.free_energy()
    assert out["converged"] and out["residual"][0] <= 1e-10
    Rg, _ = sysr.residual(x)
    assert np.linalg.norm(Rg) <= 1.5e-10
    assert np.abs(x).max() > 0.5
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)


def _bsr(rowptr, cols, vals):
    import scipy.sparse as sp

    nn = rowptr.size - 1
    return sp.bsr_matrix((vals, cols, rowptr), shape=(nn * 18, nn * 18)).tocsr()


@pytest.mark.parametrize("precision", [0, 1])
def test_periodic_multigrid_galerkin(gl, precision):
    """Coarse levels of a periodic box are periodic too: the prolongation maps free coarse
    nodes to free fine nodes and every coarse operator is P^T J P on the free nodes, with
    identity rows on the coarse periodic images."""
    import scipy.sparse as sp

    m = gl.box_mesh([-5, -5, -3], [5, 5, 3], (8, 7, 6), periodic_xy=(1, 1))
    prm = gl.Params.from_matep(P_BAR, T_RED, precond=gl.PC_MULTIGRID, precision=precision, bt=3.0)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.05, seed=4)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        f.solve(1e-2, allow_unconverged=True)
        rowptr, cols, vals, _ = f.system()
        nlev = f.mg_levels
        levels = [(rowptr, cols, vals, None)] + [f.mg_level(l) for l in range(1, nlev + 1)]
    assert nlev >= 3
    fine_mask = np.asarray(m.mask, np.uint32)
    fine_con = np.diff(m.hptr) > 0
    for l in range(1, nlev + 1):
        rp_f, c_f, v_f, _ = levels[l - 1]
        rp_c, c_c, v_c, (ptr, idx, w) = levels[l]
        nf, nc = rp_f.size - 1, rp_c.size - 1
        Pn = sp.csr_matrix((w, idx, ptr), shape=(nf, nc))
        rs = np.asarray(Pn.sum(axis=1)).ravel()
        assert np.allclose(rs[~fine_con], 1.0, atol=1e-14) and not rs[fine_con].any()
        coarse_con = np.bincount(idx, minlength=nc) == 0
        assert coarse_con.any()
        single = (np.diff(ptr) == 1) & np.isclose(w[ptr[:-1].clip(max=w.size - 1)], 1.0)
        coarse_mask = np.zeros(nc, np.uint32)
        coarse_mask[idx[ptr[:-1][single]]] = fine_mask[single]
        P = sp.kron(Pn, sp.identity(18), format="csr")
        want = (P.T @ _bsr(rp_f, c_f, v_f) @ P).toarray()
        got = _bsr(rp_c, c_c, v_c).toarray()
        dmask = ((coarse_mask[:, None] >> np.arange(18)[None, :]) & 1).astype(bool) | coarse_con[:, None]
        dmask = dmask.ravel()
        free = ~dmask
        scale = np.abs(want[np.ix_(free, free)]).max()
        # mixed mode stores the large coarse levels in FP16 (unit roundoff 4.9e-4), the others in FP32
        half = precision == 1 and nc >= 2000
        tol = 1e-13 if precision == 0 else (1e-3 if half else 2e-6)
        assert np.abs(got[np.ix_(free, free)] - want[np.ix_(free, free)]).max() <= tol * scale
        assert np.array_equal(got[dmask], np.eye(got.shape[0])[dmask])
        assert not got[np.ix_(free, dmask)].any()
        fine_mask, fine_con = coarse_mask, coarse_con


def test_periodic_multigrid_tight_solve(gl, oracle_gl):
    m = gl.box_mesh([-5, -5, -5], [5, 5, 5], (8, 8, 8), periodic_xy=(1, 1))
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=0.05, seed=3)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(gl.Params.from_matep(P_BAR, T_RED)))
    its = {}
    for name, pc in (("mg", gl.PC_MULTIGRID), ("bj", gl.PC_BLOCK_JACOBI)):
        with gl.FemGL(m, gl.Params.from_matep(P_BAR, T_RED, precond=pc)) as f:
            f.set_solution(x0)
            f.assemble_system()
            its[name] = int(f.solve(1e-10)[0])
            d = f.update()
            _, _, J, rhs = f.system()
            if name == "mg":
                assert f.mg_levels >= 2
        r = sysr.spmv(J, d) - rhs
        r[~sysr.free] = 0.0
        assert np.linalg.norm(r) <= 2e-10 * np.linalg.norm(rhs)
        assert np.allclose(sysr.distribute(d), d, rtol=0, atol=1e-14)
    assert its["mg"] < its["bj"], its


def test_pdw_start_on_periodic_slab(gl, oracle_gl):
    """The reference's weak-coupling PDW scenario: x / y periodic slab between pair-breaking z
    walls, Newton from the PDW initial state; FP64 follows the oracle's Newton path."""
    half_D = 5.0
    m = gl.box_mesh([-6.0, -6.0, -half_D], [6.0, 6.0, half_D], (6, 6, 5), periodic_xy=(1, 1))
    prm = gl.Params.from_matep(P_BAR, T_RED)
    x0 = gl.pdw_guess(P_BAR, T_RED, m.xyz, 0.3, half_D)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    # |R| reaches the FP64 floor (~1e-10 here) right after the quadratic phase: stop at 1e-9 so
    # that the iteration count is not decided by rounding
    xr, hist = oracle_gl.newton(sysr, x0, tol=1e-9, max_iter=40)
    _, Fr = sysr.residual(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        assert np.allclose(f.solution(), sysr.distribute(x0), rtol=0, atol=1e-15)
        out = f.run(max_newton=40, linear_tol=1e-12, converge_acc=1e-9)
        F = f.free_energy()
    assert out["converged"] and out["residual"][0] <= 1e-9
    assert out["newton_its"][0] == len(hist)
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)
