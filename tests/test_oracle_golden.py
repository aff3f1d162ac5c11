"""The oracle's restated per-quadrature-point physics against the reference's own
cell kernels (golden vectors generated by tests/golden/make_golden.py from the
unmodified reference sources)."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _cm(a):
    return a[:9].reshape(3, 3) + 1j * a[9:].reshape(3, 3)


def _div6(g):
    g = g.reshape(3, 18)
    return np.array([sum(g[x, 9 * part + 3 * mu + x] for x in range(3)) for part in range(2) for mu in range(3)])


@pytest.fixture(scope="module")
def kern():
    return dict(np.load(os.path.join(GOLD, "kernels.npz")))


def _unit_coef(t):
    """coefficients that isolate one bulk term: alpha (t=0) or beta_t."""
    c = np.zeros(8)
    if t == 0:
        c[2] = 1.0
    else:
        c[2 + t] = 0.5  # R = alpha A + 2 sum beta_t G_t: beta_t = 1/2 isolates G_t
    return c


def test_bulk_residual_matches_reference_kernels(oracle_gl, kern):
    for s in range(kern["A"].shape[0]):
        for t in range(6):
            R, _, _ = oracle_gl.bulk_q(_unit_coef(t), kern["A"][s])
            got = R @ kern["Pi"][s]
            ref = kern["bulk_vec"][s, t]
            assert abs(got - ref) <= 1e-13 * max(1.0, abs(ref)), (s, t, got, ref)


def test_bulk_hessian_matches_reference_kernels(oracle_gl, kern):
    for s in range(kern["A"].shape[0]):
        for t in range(6):
            _, H, _ = oracle_gl.bulk_q(_unit_coef(t), kern["A"][s])
            got = kern["Pi"][s] @ H @ kern["Pj"][s]
            ref = kern["bulk_mat"][s, t]
            assert abs(got - ref) <= 1e-13 * max(1.0, abs(ref)), (s, t, got, ref)


def test_bulk_hessian_symmetric_and_is_derivative(oracle_gl, kern):
    coef = np.array([0.42072, 0.84144, -0.4, -0.0108, 0.0206, 0.0212, 0.0198, -0.0233])
    for s in range(8):
        a = kern["A"][s]
        R0, H, _ = oracle_gl.bulk_q(coef, a)
        assert np.abs(H - H.T).max() <= 1e-14 * np.abs(H).max()
        eps = 1e-6
        for d in range(18):
            e = np.zeros(18)
            e[d] = eps
            Rp, _, _ = oracle_gl.bulk_q(coef, a + e)
            Rm, _, _ = oracle_gl.bulk_q(coef, a - e)
            assert np.allclose((Rp - Rm) / (2 * eps), H[:, d], rtol=1e-7, atol=1e-8)


def test_invariant_identity(oracle_gl, kern):
    """R(A).A = alpha tr(AA^+) + 2 sum beta_t I_t and f = alpha tr(AA^+) + sum beta_t I_t:
    the residual is the half-gradient of f (Euler: quadratic x2, quartic x4)."""
    rng = np.random.default_rng(3)
    for s in range(16):
        a = kern["A"][s]
        A = _cm(a)
        P, Q = A @ A.T, A @ A.conj().T
        inv = [abs(np.trace(P)) ** 2, np.trace(Q).real ** 2, np.trace(P @ P.conj()).real,
               np.trace(Q @ Q).real, np.trace(Q @ Q.conj()).real]
        betas = rng.standard_normal(5) * 0.02
        alpha = -0.4
        coef = np.array([0.0, 0.0, alpha, *betas])
        R, _, f = oracle_gl.bulk_q(coef, a)
        q = np.trace(Q).real
        assert np.isclose(f, alpha * q + np.dot(betas, inv), rtol=1e-12)
        assert np.isclose(R @ a, alpha * q + 2 * np.dot(betas, inv), rtol=1e-12)


def test_gradient_kernels_restated(kern):
    """K1: sum_k tr(d_kX d_kY^T) over u and v; K2K3: sum over (part, mu) of divergences."""
    for s in range(kern["A"].shape[0]):
        assert np.isclose(kern["gA"][s] @ kern["gPi"][s], kern["grad_vec"][s, 0], rtol=1e-13, atol=1e-13)
        assert np.isclose(kern["gPi"][s] @ kern["gPj"][s], kern["grad_mat"][s, 0], rtol=1e-13, atol=1e-13)
        assert np.isclose(_div6(kern["gA"][s]) @ _div6(kern["gPi"][s]), kern["grad_vec"][s, 1], rtol=1e-13,
                          atol=1e-13)
        assert np.isclose(_div6(kern["gPi"][s]) @ _div6(kern["gPj"][s]), kern["grad_mat"][s, 1], rtol=1e-13,
                          atol=1e-13)
        assert np.isclose(kern["A"][s] @ kern["Pi"][s], kern["face_vec"][s], rtol=1e-13, atol=1e-13)
        assert np.isclose(kern["Pi"][s] @ kern["Pj"][s], kern["face_mat"][s], rtol=1e-13, atol=1e-13)


def test_cell_matrix_matches_reference_loop(oracle_gl):
    """The factorised cell assembly equals the reference's per-(i,j,q) loop."""
    g = np.load(os.path.join(GOLD, "cell.npz"))
    c9 = g["coef9"]
    coef = np.array([c9[0], c9[1] + c9[2], *c9[3:]])
    K, r, _ = oracle_gl.cell_local(g["h"], g["x"], coef)
    Kref = g["cell_matrix"]
    assert np.abs(K - Kref).max() <= 1e-13 * np.abs(Kref).max()
    # reference rhs = -R
    assert np.abs(r + g["cell_rhs"]).max() <= 1e-13 * np.abs(g["cell_rhs"]).max()


def test_robin_faces_match_reference_face_loop(oracle_gl):
    """Each Robin face of the oracle's cell equals the reference's face loop (assemble.cc:286-348)."""
    g = np.load(os.path.join(GOLD, "face.npz"))
    coef = oracle_gl.coef_vector(-0.4, np.full(5, 0.01), K1=float(g["K1"]), bt=float(g["bt"]))
    K0, r0, f0 = oracle_gl.cell_local(g["h"], g["x"], coef)
    for face in range(6):
        K, r, f = oracle_gl.cell_local(g["h"], g["x"], coef, faces=1 << face)
        Kref, rref = g["face_matrix"][face], g["face_rhs"][face]
        assert np.abs(Kref).max() > 0
        assert np.abs((K - K0) - Kref).max() <= 1e-13 * np.abs(Kref).max()
        assert np.abs((r - r0) + rref).max() <= 1e-13 * np.abs(rref).max()
        # the surface energy wR |A_t|^2 has the face residual as half its gradient and is
        # homogeneous of degree 2, so x . R_face = x . dF/dx / 2 = F_face
        assert np.isclose(f - f0, (r - r0) @ g["x"].reshape(144), rtol=1e-12)
    # all six at once add up
    K6, r6, _ = oracle_gl.cell_local(g["h"], g["x"], coef, faces=63)
    assert np.abs((K6 - K0) - g["face_matrix"].sum(0)).max() <= 1e-13 * np.abs(g["face_matrix"]).max()
    # inactive when bt >= 1e10
    coef_off = oracle_gl.coef_vector(-0.4, np.full(5, 0.01), K1=float(g["K1"]))
    Koff, _, _ = oracle_gl.cell_local(g["h"], g["x"], coef_off, faces=63)
    assert np.array_equal(Koff, oracle_gl.cell_local(g["h"], g["x"], coef_off)[0])


def test_live_reference_kernels_when_built(oracle_gl):
    """With the reference tree present (this container), also compare on fresh samples."""
    R = oracle_gl.ref()
    if R is None:
        pytest.skip("reference kernels not built here")
    rng = np.random.default_rng(11)
    dp = oracle_gl._dp
    for _ in range(16):
        a, pi, pj = (rng.standard_normal(18) for _ in range(3))
        for t in range(6):
            Rq, H, _ = oracle_gl.bulk_q(_unit_coef(t), a)
            rv = R.ref_bulk_vec(t, a.ctypes.data_as(dp), pi.ctypes.data_as(dp))
            rm = R.ref_bulk_mat(t, a.ctypes.data_as(dp), pi.ctypes.data_as(dp), pj.ctypes.data_as(dp))
            assert abs(Rq @ pi - rv) <= 1e-13 * max(1, abs(rv))
            assert abs(pi @ H @ pj - rm) <= 1e-13 * max(1, abs(rm))


def test_matep_golden_self_consistent():
    d = json.load(open(os.path.join(GOLD, "matep.json")))
    row = [r for r in d["rows"] if r["p"] == 20.0 and r["t"] == 0.6 and r["scc"] == 1][0]["out"]
    # values quoted from the compiled reference Matep at p = 20 bar, t = 0.6
    assert row[0] == -0.4
    assert row[1] == -0.010867967005548968
    assert row[7] == 3.581731300383963


def _cm(a):
    return (a[:9] + 1j * a[9:]).reshape(3, 3)


def _pack(M):
    return np.concatenate([M.real.ravel(), M.imag.ravel()])


def test_hessian_vector_product_grouping(oracle_gl):
    """The matrix-free operator's closed form of H f (the grouping of its three thread groups)
    equals the oracle's bulk Hessian, which the golden kernels pin to the reference:
      alpha f + 2 b3 dG_3;  2 b1 dG_1 + [w4 (S + S^+) + w5 (conj S + S^T)] A;
      2 b2 dG_2 + (w4 Q + w5 Q^*) F,  with S = F A^+, Q = A A^+, w_t = 2 b_t."""
    rng = np.random.default_rng(21)
    H_ = lambda M: M.conj().T  # noqa: E731
    for _ in range(8):
        a, f = rng.standard_normal(18), rng.standard_normal(18)
        alpha, b = rng.standard_normal(), rng.standard_normal(5)
        coef = np.array([0.0, 0.0, alpha, *b])
        _, H, _ = oracle_gl.bulk_q(coef, a)
        ref = H.reshape(18, 18) @ f
        A, F = _cm(a), _cm(f)
        P, Q = A @ A.T, A @ H_(A)
        S3 = A @ F.T
        g0 = alpha * F + 2 * b[2] * ((S3 + S3.T) @ A.conj() + P @ F.conj())
        p, dp = np.trace(P), 2 * np.sum(A * F)
        S = F @ H_(A)
        w4, w5 = 2 * b[3], 2 * b[4]
        g1 = 2 * b[0] * (dp * A.conj() + p * F.conj()) + (w4 * (S + H_(S)) + w5 * (S.conj() + S.T)) @ A
        q, dq = np.trace(Q).real, 2 * np.sum((A.conj() * F).real)
        g2 = 2 * b[1] * (dq * A + q * F) + (w4 * Q + w5 * Q.conj()) @ F
        got = _pack(g0 + g1 + g2)
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
