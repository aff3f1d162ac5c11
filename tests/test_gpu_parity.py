"""GPU parity: the CUDA path through the C ABI against the FP64 CPU oracle.

Tolerances (FP64 mode): Jacobian and residual 1e-12 relative,
Newton iteration counts equal, converged order parameter and free energy 1e-9
relative.  Mixed mode (FP32 Jacobian/GMRES, FP64 residual): Jacobian 1e-5 relative
to the FP64 oracle, converged residual and free energy as in FP64 mode.
"""
import numpy as np
import pytest

from _lib import coef_of, oracle_mesh, product

pytestmark = pytest.mark.gpu

P_BAR, T_RED = 20.0, 0.6


@pytest.fixture(scope="module")
def gl():
    return product()


def _problem(gl, n=4, frac=0.0, half=1.25, noise=0.3, seed=7, **kw):
    m = gl.cube_mesh(half, n, frac)
    prm = gl.Params.from_matep(P_BAR, T_RED, **kw)
    x0 = gl.bphase_guess(P_BAR, T_RED, m.nn, noise=noise, seed=seed)
    return m, prm, x0


def _free_block_err(sysr, J_gpu, J_ref):
    """max |J_gpu - J_ref| over unconstrained rows/cols, relative to max |J_ref|."""
    free = sysr.free.reshape(-1, 18)
    rows = np.repeat(np.arange(sysr.m.nn), np.diff(sysr.rowptr))
    mask = free[rows][:, :, None] & free[sysr.cols][:, None, :]
    d = np.where(mask, J_gpu - J_ref, 0.0)
    return np.abs(d).max() / np.abs(np.where(mask, J_ref, 0.0)).max()


@pytest.mark.parametrize("n,frac", [(4, 0.0), (4, 0.25), (5, 0.2)])
def test_assembly_fp64_matches_oracle(gl, oracle_gl, n, frac):
    m, prm, x0 = _problem(gl, n, frac)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        rn = f.assemble_system()
        rowptr, cols, J, rhs = f.system()
        x = f.solution()
    xr = sysr.distribute(x0)
    assert np.allclose(x, xr, rtol=0, atol=1e-15)
    Jr, Rr, Fr = sysr.assemble(xr)
    assert np.array_equal(rowptr, sysr.rowptr) and np.array_equal(cols, sysr.cols)
    assert _free_block_err(sysr, J, Jr) <= 1e-12
    assert np.abs(rhs + Rr).max() <= 1e-12 * np.abs(Rr).max()
    assert np.all(rhs[~sysr.free] == 0.0)
    assert abs(rn[0] - np.linalg.norm(Rr)) <= 1e-12 * np.linalg.norm(Rr)


def test_residual_energy_spmv_fp64(gl, oracle_gl):
    m, prm, x0 = _problem(gl, 4, 0.25)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr = sysr.distribute(x0)
    Jr, Rr, Fr = sysr.assemble(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        nr = f.compute_residual()
        R = f.residual()
        F = f.free_energy()
        f.assemble_system()
        v = np.random.default_rng(1).standard_normal(sysr.nd)
        y = f.spmv(v)
    assert np.abs(R - Rr).max() <= 1e-12 * np.abs(Rr).max()
    assert abs(nr[0] - np.linalg.norm(Rr)) <= 1e-12 * np.linalg.norm(Rr)
    assert abs(F[0] - Fr) <= 1e-12 * abs(Fr)
    yr = sysr.spmv(Jr, v)
    # constrained rows carry only a diagonal whose value is a convention (deal.II writes
    # a cell-summed |diagonal|); every unconstrained row must agree
    fr = sysr.free
    assert np.abs(y - yr)[fr].max() <= 1e-12 * np.abs(yr[fr]).max()


def test_assembly_mixed_fp32_jacobian(gl, oracle_gl):
    m, prm, x0 = _problem(gl, 4, 0.25, precision=gl.MIXED)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr = sysr.distribute(x0)
    Jr, Rr, _ = sysr.assemble(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        _, _, J, rhs = f.system()
    assert _free_block_err(sysr, J, Jr) <= 1e-5
    # the residual stays FP64 in mixed mode
    assert np.abs(rhs + Rr).max() <= 1e-12 * np.abs(Rr).max()


@pytest.mark.parametrize("refine", [0.25, 0.0])
def test_spmv_mixed_matrix_free(gl, oracle_gl, refine):
    # mixed mode applies J matrix-free from the FP32 quadrature Hessians; on every
    # unconstrained row it must equal the assembled FP32 matrix and the oracle's FP64 J
    m, prm, x0 = _problem(gl, 4, refine, precision=gl.MIXED)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    Jr, _, _ = sysr.assemble(sysr.distribute(x0))
    v = np.random.default_rng(7).standard_normal(18 * m.nn)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        y = f.spmv(v)
        _, _, J, _ = f.system()
    fr = sysr.free
    v32 = v.astype(np.float32).astype(np.float64)
    y_bsr = sysr.spmv(J, v32)
    y_ref = sysr.spmv(Jr, v32)
    scale = np.abs(y_ref[fr]).max()
    assert np.abs(y - y_bsr)[fr].max() <= 2e-5 * scale
    assert np.abs(y - y_ref)[fr].max() <= 2e-5 * scale


@pytest.mark.parametrize("precond", ["bj", "cheb", "none"])
def test_linear_solve_tight(gl, oracle_gl, precond):
    pc = {"bj": gl.PC_BLOCK_JACOBI, "cheb": gl.PC_CHEBYSHEV, "none": gl.PC_NONE}[precond]
    m, prm, x0 = _problem(gl, 4, 0.25, precond=pc, noise=0.05)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        its = f.solve(1e-10)
        d = f.update()
        _, _, J, rhs = f.system()
    assert its[0] > 0
    r = sysr.spmv(J, d) - rhs
    r[~sysr.free] = 0.0
    assert np.linalg.norm(r) <= 2e-10 * np.linalg.norm(rhs)
    # delta satisfies the constraints (Dirichlet zeros, hanging = parent average)
    assert np.allclose(sysr.distribute(d), d, rtol=0, atol=1e-14)


def test_newton_fp64_matches_oracle(gl, oracle_gl):
    m, prm, x0 = _problem(gl, 4, 0.0, half=2.5, noise=0.05, seed=2)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr, hist = oracle_gl.newton(sysr, x0, tol=1e-10, max_iter=40)
    _, Fr = sysr.residual(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        out = f.run(max_newton=40, linear_tol=1e-12, converge_acc=1e-10)
        x = f.solution()
        F = f.free_energy()
    assert out["converged"]
    assert out["newton_its"][0] == len(hist)
    assert out["residual"][0] <= 1e-10
    assert np.abs(x - xr).max() <= 1e-9 * np.abs(xr).max()
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)


def test_newton_step_by_step_matches_oracle(gl, oracle_gl):
    """The reference's per-step calls: assemble, solve, newton_iteration."""
    m, prm, x0 = _problem(gl, 4, 0.25, half=2.5, noise=0.1, seed=3)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    hist_r = []
    oracle_gl.newton(sysr, x0, tol=1e-10, max_iter=3, log=hist_r.append)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        for step in range(min(3, len(hist_r))):
            rn = f.assemble_system()
            f.solve(1e-12)
            res, trials = f.newton_iteration()
            h = hist_r[step]
            assert abs(rn[0] - h["res_before"]) <= 1e-9 * h["res_before"]
            assert trials[0] == h["trials"]
            assert abs(res[0] - h["res"]) <= 1e-8 * h["res_before"] + 1e-13


def test_newton_mixed_reaches_fp64_answer(gl, oracle_gl):
    m, prm, x0 = _problem(gl, 4, 0.25, half=2.5, noise=0.05, seed=2, precision=gl.MIXED)
    sysr = oracle_gl.System(oracle_mesh(m), coef_of(prm))
    xr, hist = oracle_gl.newton(sysr, x0, tol=1e-10, max_iter=40)
    _, Fr = sysr.residual(xr)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        out = f.run(max_newton=60, linear_tol=1e-4, converge_acc=1e-10)
        x = f.solution()
        F = f.free_energy()
    assert out["converged"] and out["residual"][0] <= 1e-10
    # the converged residual is FP64: check it on the oracle too
    Rg, _ = sysr.residual(x)
    assert np.linalg.norm(Rg) <= 1.5e-10
    assert abs(F[0] - Fr) <= 1e-9 * abs(Fr)


def test_batched_instances_match_single(gl):
    meshes = [gl.cube_mesh(2.5, 3), gl.cube_mesh(2.0, 4, 0.25), gl.box_mesh([-1, -2, -1.5], [1, 2, 1.5], (3, 4, 3))]
    pts = [(20.0, 0.6), (10.0, 0.5), (30.0, 0.8)]
    prms = [gl.Params.from_matep(p, t) for p, t in pts]
    x0s = [gl.bphase_guess(p, t, m.nn, noise=0.05, seed=k) for k, (m, (p, t)) in enumerate(zip(meshes, pts))]
    singles = []
    for m, prm, x0 in zip(meshes, prms, x0s):
        with gl.FemGL(m, prm) as f:
            f.set_solution(x0)
            o = f.run(max_newton=40, linear_tol=1e-12, converge_acc=1e-10)
            singles.append((o, f.solution(), f.free_energy()[0]))
    with gl.FemGL(meshes, prms) as f:
        f.set_solution(np.concatenate(x0s))
        o = f.run(max_newton=40, linear_tol=1e-12, converge_acc=1e-10)
        xb = f.solution()
        Fb = f.free_energy()
    off = np.cumsum([0] + [18 * m.nn for m in meshes])
    for k, (os_, xs, Fs) in enumerate(singles):
        assert o["newton_its"][k] == os_["newton_its"][0]
        assert np.abs(xb[off[k]:off[k + 1]] - xs).max() <= 1e-10 * np.abs(xs).max()
        assert abs(Fb[k] - Fs) <= 1e-10 * abs(Fs)


@pytest.mark.parametrize("n,L", [(16, 1.0), (24, 10.0), (64, 1.0), (64, 10.0)])
def test_complexgl_2d_matches_oracle(gl, oracle_gl, n, L):
    """complexGL 2D: the benchmark configuration (64 x 64 Q1 on the unit square, where
    the normal state psi = 0 is the stable solution), smaller grids, and L = 10, where
    the ordered state |psi|^2 = -alpha/beta forms."""
    from oracle import mesh as om

    m = gl.square_mesh(n, L)
    prm = gl.Params(alpha=-1.0, beta=[0.5, 0, 0, 0, 0], K1=1.0)
    rng = np.random.default_rng(1)
    x0 = 1.0 + 0.1 * rng.uniform(-1, 1, 2 * m.nn)
    sysr = oracle_gl.System2D(om.square_mesh(n, L), alpha=-1.0, beta=0.5, K=1.0)
    xr0 = sysr.distribute(x0)
    Jr, Rr, Fr = sysr.assemble(xr0)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        rowptr, cols, J, rhs = f.system()
        import scipy.sparse as sp

        Jg = sp.bsr_matrix((J, cols, rowptr), shape=(2 * m.nn, 2 * m.nn)).toarray()
        fr = sysr.free
        Jd = Jr.toarray()
        err = np.abs((Jg - Jd)[np.ix_(fr, fr)]).max() / np.abs(Jd).max()
        assert err <= 1e-12
        assert np.abs(rhs + Rr).max() <= 1e-12 * np.abs(Rr).max()
        out = f.run(max_newton=40, linear_tol=1e-12, converge_acc=1e-10)
        F = f.free_energy()
        x = f.solution()
    # oracle Newton with the same reference semantics
    xo = xr0.copy()
    for it in range(41):
        J_, R_, _ = sysr.assemble(xo)
        prev = np.linalg.norm(R_)
        d = sysr.solve_exact(J_, -R_)
        for i in range(100):
            xt = sysr.distribute(xo + 0.83 ** i * d)
            cur = np.linalg.norm(sysr.residual(xt)[0])
            if cur < prev:
                break
        xo = xt
        if cur <= 1e-10:
            break
    _, Fo = sysr.residual(xo)
    assert out["converged"] and out["newton_its"][0] == it + 1
    # psi -> e^{i phi} psi is an exact symmetry (the psi = 0 edge keeps it), so the two
    # Newton runs may stop at different points of the same orbit: compare after the phase
    # that best aligns them
    psi, ref = x[0::2] + 1j * x[1::2], xo[0::2] + 1j * xo[1::2]
    psi = psi * np.exp(1j * np.angle(np.vdot(psi, ref)))
    xa = np.stack([psi.real, psi.imag], axis=1).ravel()
    assert np.abs(xa - xo).max() <= 1e-9 * max(1.0, np.abs(xo).max()), np.abs(xa - xo).max()
    assert abs(F[0] - Fo) <= 1e-9 * max(1.0, abs(Fo))
    if L > 1.0:
        # ordered bulk: |psi|^2 -> -alpha/beta = 2 away from the Dirichlet edge
        psi2 = x[0::2] ** 2 + x[1::2] ** 2
        assert abs(psi2.max() - 2.0) < 0.05


def test_state_errors(gl):
    m, prm, x0 = _problem(gl, 3)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        with pytest.raises(gl.GLGPUError) as e:
            f.solve(1e-6)
        assert e.value.status == 7
        bad = x0.copy()
        free_node = int(np.flatnonzero(m.mask == 0)[0])
        bad[18 * free_node] = np.nan
        f.set_solution(bad)
        with pytest.raises(gl.GLGPUError) as e:
            f.compute_residual()
        assert e.value.status == 5
        assert f.launch_count > 0


def test_pinned_host_arrays(gl):
    """Page-locked host arrays from the library give the same copies as ordinary ones."""
    m, prm, x0 = _problem(gl, 3, 0.0)
    with gl.FemGL(m, prm) as f:
        xin = gl.pinned_array(f.n_dofs)
        xin[:] = x0
        f.set_solution(xin)
        a = f.solution()
        out = gl.pinned_array(f.n_dofs)
        b = f.solution(out=out)
        assert b is out and np.array_equal(a, b)
        f.set_solution(x0)
        assert np.array_equal(f.solution(), a)
        with pytest.raises(ValueError):
            f.solution(out=np.zeros(3))
    del xin, out  # the allocations are released with their arrays
