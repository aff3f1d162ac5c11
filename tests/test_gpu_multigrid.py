"""Geometric multigrid preconditioner (flexible GMRES) on the GPU: the coarse Jacobians
are the Galerkin products P^T J P of the level above, tight linear solves agree with the
oracle's Jacobian, Newton with multigrid reproduces the oracle's answer, batched
instances of different sizes work, and once-refined boxes (hanging nodes) get their
unrefined grid as first coarse level."""
import numpy as np
import pytest
import scipy.sparse as sp

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


def _bsr(rowptr, cols, vals):
    nn = rowptr.size - 1
    return sp.bsr_matrix((vals, cols, rowptr), shape=(nn * 18, nn * 18)).tocsr()


@pytest.mark.parametrize("precision", [0, 1])
def test_galerkin_coarse_operators(gl, precision):
    # anisotropic slab with an odd cell count: semi-coarsening and an uneven last line
    m = gl.box_mesh([-10, -10, -4], [10, 10, 4], (9, 9, 9))
    prm = gl.Params.from_matep(20.0, 0.6, precond=gl.PC_MULTIGRID, precision=precision)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=4)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        f.solve(1e-2, allow_unconverged=True)  # the hierarchy is built by the solve's setup
        rowptr, cols, vals, _ = f.system()
        levels = [(rowptr, cols, vals, None)] + [f.mg_level(l) for l in range(1, f.mg_levels + 1)]
        nlev = f.mg_levels
    assert nlev >= 3
    fine_mask = np.asarray(m.mask, np.uint32)
    for l in range(1, nlev + 1):
        rp_f, c_f, v_f, _ = levels[l - 1]
        rp_c, c_c, v_c, (ptr, idx, w) = levels[l]
        nf, nc = rp_f.size - 1, rp_c.size - 1
        Pn = sp.csr_matrix((w, idx, ptr), shape=(nf, nc))
        # partition of unity; every coarse node coincides with one fine node (nested grids)
        assert np.allclose(np.asarray(Pn.sum(axis=1)).ravel(), 1.0, atol=1e-14)
        single = (np.diff(ptr) == 1) & np.isclose(w[ptr[:-1].clip(max=w.size - 1)], 1.0)
        assert np.bincount(idx[ptr[:-1][single]], minlength=nc).min() == 1
        coarse_mask = np.zeros(nc, np.uint32)
        coarse_mask[idx[ptr[:-1][single]]] = fine_mask[single]
        P = sp.kron(Pn, sp.identity(18), format="csr")
        want = (P.T @ _bsr(rp_f, c_f, v_f) @ P).toarray()
        got = _bsr(rp_c, c_c, v_c).toarray()
        dmask = ((coarse_mask[:, None] >> np.arange(18)[None, :]) & 1).astype(bool).ravel()
        free = ~dmask
        scale = np.abs(want[np.ix_(free, free)]).max()
        # mixed mode stores the large coarse levels in FP16 (unit roundoff 4.9e-4), the others in FP32
        half = precision == 1 and nc >= 2000
        tol = 1e-13 if precision == 0 else (1e-3 if half else 2e-6)
        assert np.abs(got[np.ix_(free, free)] - want[np.ix_(free, free)]).max() <= tol * scale
        # constrained components: identity rows, zero columns
        assert np.array_equal(got[dmask], np.eye(got.shape[0])[dmask])
        assert not got[np.ix_(free, dmask)].any()
        fine_mask = coarse_mask


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


@pytest.mark.parametrize("precision", [0, 1])
def test_multigrid_on_refined_mesh(gl, oracle_gl, precision):
    """A once-refined box (hanging nodes on the coarse-fine faces) gets multigrid with its
    unrefined grid as first coarse level: that level's Jacobian is P^T J P over the free fine
    nodes, and a tight solve satisfies the Jacobian in fewer iterations than block-Jacobi."""
    m = gl.box_mesh([-5.0, -5.0, -5.0], [5.0, 5.0, 5.0], (8, 8, 8), refine_band=1.5)
    assert m.n_hanging > 0
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=3)
    tol = 1e-10 if precision == 0 else 1e-8
    res = {}
    for pc in (gl.PC_MULTIGRID, gl.PC_BLOCK_JACOBI):
        prm = gl.Params.from_matep(20.0, 0.6, precond=pc, precision=precision)
        with gl.FemGL(m, prm) as f:
            f.set_solution(x0)
            f.assemble_system()
            its = f.solve(tol, allow_unconverged=pc == gl.PC_BLOCK_JACOBI)
            res[pc] = (int(its[0]), f.update(), f.system(), f.mg_levels,
                       f.mg_level(1) if pc == gl.PC_MULTIGRID else None)
    its_mg, d, (rowptr, cols, vals, rhs), lev, (rp_c, c_c, v_c, (ptr, idx, w)) = res[gl.PC_MULTIGRID]
    assert lev >= 3 and res[gl.PC_BLOCK_JACOBI][3] == 0
    nf, nc = rowptr.size - 1, rp_c.size - 1
    assert nc == 9 ** 3
    hang = np.diff(np.asarray(m.hptr)) > 0
    assert np.array_equal(np.diff(ptr) == 0, hang)
    Pn = sp.csr_matrix((w, idx, ptr), shape=(nf, nc))
    P = sp.kron(Pn, sp.identity(18), format="csr")
    want = (P.T @ _bsr(rowptr, cols, vals) @ P).tocsr()
    got = _bsr(rp_c, c_c, v_c)
    single = (np.diff(ptr) == 1) & np.isclose(w[ptr[:-1].clip(max=w.size - 1)], 1.0)
    assert np.bincount(idx[ptr[:-1][single]], minlength=nc).min() == 1
    cmask = np.zeros(nc, np.uint32)
    cmask[idx[ptr[:-1][single]]] = np.asarray(m.mask, np.uint32)[single]
    free = ~((((cmask[:, None] >> np.arange(18)[None, :]) & 1) != 0).ravel())
    Df = sp.diags(free.astype(float))
    diff = (Df @ (want - got) @ Df).tocsr()
    scale = np.abs((Df @ want @ Df).data).max()
    assert np.abs(diff.data).max() <= (1e-13 if precision == 0 else 2e-6) * scale
    # the solve: residual of the assembled Jacobian over the free fine rows
    fr = np.repeat((np.asarray(m.mask) == 0) & ~hang, 18)
    r = _bsr(rowptr, cols, vals) @ d - rhs
    assert np.linalg.norm(r[fr]) <= (2e-10 if precision == 0 else 2e-5) * np.linalg.norm(rhs)
    assert its_mg < res[gl.PC_BLOCK_JACOBI][0], (its_mg, res[gl.PC_BLOCK_JACOBI][0])


def test_newton_multigrid_refined_matches_fp64(gl):
    """Mixed-precision multigrid Newton on a refined box reaches the FP64 block-Jacobi
    Newton's minimum: same free energy, |F| < 1e-10, and the same |A|^2 at every node.
    Spin rotations and the global phase are exact symmetries with natural x / y faces, so
    the two solvers may stop at different points of the same orbit: states are compared
    through the invariant."""
    m = gl.box_mesh([-5.0, -5.0, -4.0], [5.0, 5.0, 4.0], (8, 8, 6), refine_band=1.5)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=2)
    out = {}
    for name, prec, pc, ltol in (("mg", gl.MIXED, gl.PC_MULTIGRID, 1e-4), ("ref", gl.FP64, gl.PC_BLOCK_JACOBI, 1e-12)):
        prm = gl.Params.from_matep(20.0, 0.6, precision=prec, precond=pc)
        with gl.FemGL(m, prm) as f:
            f.set_solution(x0)
            o = f.run(max_newton=40, linear_tol=ltol, converge_acc=1e-10)
            out[name] = (o, f.free_energy()[0], f.solution(), f.mg_levels, f.mg_fallbacks)
    om, Fm, xm, lev, fb = out["mg"]
    orf, Fr, xr, _, _ = out["ref"]
    assert om["converged"] and orf["converged"] and lev >= 2 and fb == 0
    assert om["residual"][0] <= 1e-10
    assert abs(Fm - Fr) <= 1e-9 * abs(Fr)
    am, ar = (xm.reshape(-1, 18) ** 2).sum(1), (xr.reshape(-1, 18) ** 2).sum(1)
    assert np.abs(am - ar).max() <= 1e-6 * ar.max()


def test_preconditioner_reuse(gl):
    # keeping the previous step's multigrid hierarchy for small Newton steps changes the
    # Krylov path only: same Newton history and free energy; and the block matrix, not
    # re-assembled on such steps, is rebuilt when it is read
    m = gl.cube_mesh(5.0, 8)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=2)
    res = {}
    for reuse in (0.0, 1e-2):
        prm = gl.Params.from_matep(20.0, 0.6, precision=gl.MIXED, precond=gl.PC_MULTIGRID, prec_reuse=reuse)
        with gl.FemGL(m, prm) as f:
            f.set_solution(x0)
            out = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
            x, F = f.solution(), f.free_energy()[0]
            f.assemble_system()
            _, _, J, _ = f.system()
        res[reuse] = (out, x, F, J)
    o0, x0r, F0, _ = res[0.0]
    o1, x1, F1, J1 = res[1e-2]
    assert o0["converged"] and o1["converged"]
    assert o1["newton_its"][0] == o0["newton_its"][0]
    assert abs(F1 - F0) <= 1e-12 * abs(F0)
    prm = gl.Params.from_matep(20.0, 0.6, precision=gl.MIXED, precond=gl.PC_MULTIGRID)
    with gl.FemGL(m, prm) as g:
        g.set_solution(x1)
        g.assemble_system()
        _, _, Jf, _ = g.system()
    assert np.array_equal(J1, Jf)


def test_galerkin_fp16_level(gl):
    """Mixed mode stores coarse levels with >= 2000 nodes in FP16: level 1 of a 24^3 grid
    (13^3 nodes) equals P^T J P to FP16 rounding, identity rows stay exact, and the solve
    still reaches a tight tolerance through flexible GMRES."""
    m = gl.cube_mesh(7.5, 24)
    prm = gl.Params.from_matep(20.0, 0.6, precond=gl.PC_MULTIGRID, precision=gl.MIXED)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=4)
    with gl.FemGL(m, prm) as f:
        f.set_solution(x0)
        f.assemble_system()
        its = f.solve(1e-8)
        rowptr, cols, vals, rhs = f.system()
        d = f.update()
        rp_c, c_c, v_c, (ptr, idx, w) = f.mg_level(1)
    nf, nc = rowptr.size - 1, rp_c.size - 1
    assert nc == 13 ** 3
    Pn = sp.csr_matrix((w, idx, ptr), shape=(nf, nc))
    P = sp.kron(Pn, sp.identity(18), format="csr")
    want = (P.T @ _bsr(rowptr, cols, vals) @ P).tocsr()
    got = _bsr(rp_c, c_c, v_c)
    single = (np.diff(ptr) == 1) & np.isclose(w[ptr[:-1].clip(max=w.size - 1)], 1.0)
    cmask = np.zeros(nc, np.uint32)
    cmask[idx[ptr[:-1][single]]] = np.asarray(m.mask, np.uint32)[single]
    free = ~((((cmask[:, None] >> np.arange(18)[None, :]) & 1) != 0).ravel())
    Df = sp.diags(free.astype(float))
    diff = (Df @ (want - got) @ Df).tocsr()
    scale = np.abs((Df @ want @ Df).data).max()
    assert np.abs(diff.data).max() <= 1e-3 * scale
    assert np.abs(diff.data).max() > 0  # really stored in FP16
    # a tight solve with the FP16 level inside the preconditioner: checked against the assembled
    # FP32 matrix, which agrees with the matrix-free operator to FP32 rounding
    r = _bsr(rowptr, cols, vals) @ d - rhs
    fr = np.repeat(np.asarray(m.mask) == 0, 18)  # interior nodes carry no constrained component
    assert int(its[0]) > 0 and np.linalg.norm(r[fr]) <= 2e-5 * np.linalg.norm(rhs)


def test_programmatic_launch_gives_identical_solves(gl):
    """Programmatic dependent launch changes only when CTAs are scheduled: every kernel
    waits on the device for its predecessor before touching memory, so the mixed
    multigrid solve (V-cycle graph, matrix-free operator, in-kernel reductions) is
    bitwise the same with it on and off."""
    m = gl.cube_mesh(5.0, 10)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=3)
    prm = gl.Params.from_matep(20.0, 0.6, precision=gl.MIXED, precond=gl.PC_MULTIGRID)
    out = {}
    try:
        for mode in (True, False):
            gl.set_launch_mode(mode)
            with gl.FemGL(m, prm) as f:
                f.set_solution(x0)
                o = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
                out[mode] = (o, f.solution())
    finally:
        gl.set_launch_mode(True)
    (o1, x1), (o0, x0b) = out[True], out[False]
    assert o1["converged"] and o0["converged"]
    assert np.array_equal(o1["newton_its"], o0["newton_its"]) and np.array_equal(o1["gmres_its"], o0["gmres_its"])
    assert np.array_equal(x1, x0b)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("precision,n_inst", [("mixed", 1), ("mixed", 3), ("fp64", 1)])
def test_fused_small_levels_match_separate_launches(gl, oracle_gl, precision, n_inst, mode):
    """The small coarse levels in fewer launches: mode 1 the levels below 20,000 nodes as one
    cooperative launch per V-cycle, mode 2 the levels of at most 160 nodes per instance and the
    dense solve as one cluster launch per instance.  The Newton solve reaches the same free
    energy and state (up to the exact symmetries) as with one launch per sweep and transfer,
    with iteration counts within one or two, and launches fewer kernels per GMRES iteration."""
    prec = gl.MIXED if precision == "mixed" else gl.FP64
    meshes = [gl.cube_mesh(5.0, 12), gl.box_mesh([-4, -4, -3], [4, 4, 3], (10, 10, 8)), gl.cube_mesh(4.0, 8)][:n_inst]
    pts = [(20.0, 0.6), (10.0, 0.5), (30.0, 0.8)][:n_inst]
    x0 = np.concatenate([gl.bphase_guess(p, t, m.nn, noise=0.05, seed=5 + k) for k, (m, (p, t)) in enumerate(zip(meshes, pts))])
    res = {}
    for fuse in (0, mode):
        prms = [gl.Params.from_matep(p, t, precision=prec, precond=gl.PC_MULTIGRID, mg_small_fuse=fuse) for p, t in pts]
        with gl.FemGL(meshes, prms) as f:
            assert f.mg_levels >= 2
            f.set_solution(x0)
            o = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
            res[fuse] = (o, f.solution(), f.free_energy(), f.mg_fallbacks, f.launch_count)
    (o0, x_0, F0, _, n0), (o1, x_1, F1, fb1, n1) = res[0], res[mode]
    assert o0["converged"] and o1["converged"] and fb1 == 0
    assert n1 / o1["gmres_its"].sum() < n0 / o0["gmres_its"].sum()
    assert np.all(np.abs(o1["gmres_its"] - o0["gmres_its"]) <= 2 + 0.1 * o0["gmres_its"])
    assert np.allclose(F1, F0, rtol=1e-9, atol=0)
    off = np.cumsum([0] + [18 * m.nn for m in meshes])
    for k in range(n_inst):
        a, b = x_1[off[k]:off[k + 1]], x_0[off[k]:off[k + 1]]
        xa, _, _ = oracle_gl.gauge_align(a, b)
        assert np.abs(xa - b).max() <= 1e-7 * np.abs(b).max()


def test_stalled_instance_handed_off_and_finished(gl):
    """A slab of the phase-diagram sweep (19^3 cells, T = 0.544 Tc, p = 11.8 bar, D = 39.1 xi0)
    whose mixed-precision multigrid solve stalls: batched with an easy instance and handoff on,
    it leaves the batch at the state it reached (flagged, unconverged) while the other converges
    unchanged; the sweep finishes it alone (stronger smoothing, then FP64), at the free energy of
    an FP64 multigrid solve from its start."""
    sweep = __import__("importlib").import_module("verkko-hem-repo_gb300.sweep")
    t, p, D, n = 0.5444804785663939, 11.833486443002236, 39.11806936676019, 19
    hard = gl.box_mesh([-10.0, -10.0, -D / 2], [10.0, 10.0, D / 2], (n, n, n))
    easy = gl.box_mesh([-10.0, -10.0, -6.0], [10.0, 10.0, 6.0], (16, 16, 16))
    xh = gl.bphase_guess(p, t, hard.nn, noise=0.05, seed=1016)
    xe = gl.bphase_guess(20.0, 0.6, easy.nn, noise=0.05, seed=7)
    prms = [gl.Params.from_matep(p, t, precision=gl.MIXED, precond=gl.PC_MULTIGRID),
            gl.Params.from_matep(20.0, 0.6, precision=gl.MIXED, precond=gl.PC_MULTIGRID)]
    with gl.FemGL([hard, easy], prms) as f:
        f.set_mg_handoff(True)
        f.set_solution(np.concatenate([xh, xe]))
        o = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10, allow_unconverged=True)
        handed = f.handed_off
        assert handed.tolist() == [True, False] and f.mg_fallbacks == 0
        assert o["residual"][0] > 1e-10 and o["residual"][1] <= 1e-10
    with gl.FemGL(easy, prms[1]) as g:
        g.set_solution(xe)
        oe = g.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        assert int(oe["newton_its"][0]) == int(o["newton_its"][1])
    r = sweep.solve_sweep(gl, [hard, easy], prms, [xh, xe])
    assert r["converged"].all() and r["handed_off"].tolist() == [True, False]
    with gl.FemGL(hard, gl.Params.from_matep(p, t, precision=gl.FP64, precond=gl.PC_MULTIGRID)) as h:
        h.set_solution(xh)
        h.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        F64 = float(h.free_energy()[0])
    assert abs(r["free_energy"][0] - F64) <= 1e-9 * abs(F64)


@pytest.mark.parametrize("precision", [0, 1])
def test_one_projection_gram_schmidt(gl, precision):
    """GMRES with one Gram-Schmidt projection per iteration (no reorthogonalization) reaches
    the same converged state and free energy, with iteration counts close to the default."""
    m = gl.cube_mesh(5.0, 12)
    x0 = gl.bphase_guess(20.0, 0.6, m.nn, noise=0.05, seed=5)
    prm = gl.Params.from_matep(20.0, 0.6, precision=precision, precond=gl.PC_MULTIGRID)
    res = {}
    for reorth in (True, False):
        with gl.FemGL(m, prm) as f:
            f.set_reorthogonalization(reorth)
            f.set_solution(x0)
            o = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
            res[reorth] = (o, f.free_energy()[0])
    (o1, F1), (o0, F0) = res[True], res[False]
    assert o1["converged"] and o0["converged"]
    assert abs(F0 - F1) <= 1e-12 * abs(F1)
    assert abs(int(o0["gmres_its"][0]) - int(o1["gmres_its"][0])) <= 2 + 0.2 * int(o1["gmres_its"][0])


@pytest.mark.parametrize("precision", [0, 1])
def test_coarsest_dense_inverse(gl, precision):
    """The coarsest level's dense inverse (in-place Gauss-Jordan with partial pivoting, one CTA
    per instance, rows held in registers) inverts that level's shifted Galerkin matrix for
    every instance of a batch: small normwise residual and agreement with an FP64 inverse."""
    meshes = [gl.box_mesh([-10, -10, -4], [10, 10, 4], (9, 9, 9)), gl.cube_mesh(5.0, 6),
              gl.box_mesh([-10, -10, -12], [10, 10, 12], (12, 12, 12))]
    pts = [(20.0, 0.6), (12.0, 0.45), (30.0, 0.85)]
    x0 = np.concatenate([gl.bphase_guess(p, t, m.nn, noise=0.05, seed=k) for k, (m, (p, t)) in
                         enumerate(zip(meshes, pts))])
    prms = [gl.Params.from_matep(p, t, precond=gl.PC_MULTIGRID, precision=precision) for p, t in pts]
    with gl.FemGL(meshes, prms) as f:
        f.set_solution(x0)
        f.assemble_system()
        f.solve(1e-2, allow_unconverged=True)  # the hierarchy and the inverses are built by the setup
        nl = f.mg_levels
        rp, cols, vals, _ = f.mg_level(nl)
        invs = [f.mg_coarse_inverse(k) for k in range(len(meshes))]
    A = _bsr(rp, cols, vals).toarray()
    assert sum(x.shape[0] for x in invs) == A.shape[0]
    off = 0
    for inv in invs:
        nd = inv.shape[0]
        assert nd % 18 == 0 and 0 < nd <= 144
        # instances are independent: the level matrix is block diagonal over them
        assert not A[off:off + nd, :off].any() and not A[off:off + nd, off + nd:].any()
        M = A[off:off + nd, off:off + nd].astype(np.float32).astype(np.float64)
        s = np.float32(prms[0].mg_coarse_shift) * np.abs(np.diag(M)).astype(np.float32).sum() / np.float32(nd)
        M += float(s) * np.eye(nd)
        X = inv.astype(np.float64)
        assert np.isfinite(X).all() and not np.array_equal(X, np.eye(nd))  # no zero pivot met
        res = np.linalg.norm(M @ X - np.eye(nd)) / (np.linalg.norm(M) * np.linalg.norm(X))
        assert res < 1e-5, res
        Xr = np.linalg.inv(M)
        # FP32 elimination: forward error within a few ulps times the condition number
        err = np.linalg.norm(X - Xr) / np.linalg.norm(Xr)
        assert err < 1e-5 * np.linalg.cond(M), (err, np.linalg.cond(M))
        off += nd
