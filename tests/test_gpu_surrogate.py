"""The surrogate network's tcgen05 kernels against the CPU oracle (oracle/mlp.py):
forward values, loss and parameter gradients, and a training run that must reduce
the loss.  Tolerances reflect BF16 activations: 1e-2 relative on outputs and on each
layer's gradient norm-wise."""
import numpy as np
import pytest

from _lib import product

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gl():
    return product()


def _inputs(n, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1, 1, (n, 6)).astype(np.float32)


def test_forward_matches_oracle(gl):
    from oracle import mlp

    with gl.Surrogate(seed=3) as s:
        X = _inputs(300)
        Y = s.predict(X)
        Yr, _, _ = mlp.forward(s.params(), X)
    assert Y.shape == (300, 18)
    err = np.abs(Y - Yr).max() / np.abs(Yr).max()
    assert err <= 1e-2, err


def test_gradient_matches_oracle(gl):
    from oracle import mlp

    rng = np.random.default_rng(1)
    X = _inputs(1000, 2)
    T = rng.standard_normal((1000, 18)).astype(np.float32)
    with gl.Surrogate(seed=5) as s:
        loss, g = s.gradient(X, T)
        lr, gr = mlp.gradient(s.params(), X, T)
    assert abs(loss - lr) <= 1e-3 * abs(lr)
    o = 0
    for fi, fo in mlp.LAYERS:
        for n in (fi * fo, fo):
            a, b = g[o:o + n], gr[o:o + n]
            assert np.linalg.norm(a - b) <= 1e-2 * np.linalg.norm(b) + 1e-12, (fi, fo, n)
            o += n


def test_training_reduces_loss(gl):
    # a smooth target of the kind the solver produces: profiles across a slab
    rng = np.random.default_rng(4)
    X = rng.uniform(-1, 1, (8192, 6)).astype(np.float32)
    T = np.zeros((8192, 18), np.float32)
    T[:, 0] = T[:, 4] = 1.0 - 0.3 * X[:, 2] ** 2
    T[:, 8] = np.tanh(3 * (1 - np.abs(X[:, 2]))) * (0.5 + 0.5 * X[:, 3])
    with gl.Surrogate(seed=0) as s:
        l0, _ = s.gradient(X[:2048], T[:2048])
        lf = s.train(X, T, steps=600, batch=2048, lr=2e-3, seed=1)
        Y = s.predict(X[:512])
    assert lf < 0.05 * l0, (l0, lf)
    assert np.abs(Y - T[:512]).max() < 0.15


def test_learned_guess_speeds_up_newton(gl):
    """Trained on converged slab states, the surrogate start needs fewer Newton steps and
    fewer GMRES iterations in total than the B-phase start (+0.05 N(0,1), the benchmark
    configurations' start) on held-out (t, p, D) instances, takes less device time, and
    reaches the same converged free energy (the plain-Newton fallback covers any failure)."""
    import importlib

    L = importlib.import_module("verkko-hem-repo_gb300.learned")
    X, Y, info = L.generate(gl, 24, seed=11, n_lo=8, n_hi=10, per_instance=1024)
    s, tinfo = L.train(gl, X, Y, steps=1500, batch=4096, lr=1e-3, seed=0)
    assert tinfo["components_kept"] < 18  # the symmetry zeros of the training states
    test = L.sample(gl, 4, seed=99, n_lo=10, n_hi=12)
    L.solve(gl, test, L.bphase_starts(gl, test, 0.05, 5), gl.MIXED)  # warm-up
    _, ob, ms_b = L.solve(gl, test, L.bphase_starts(gl, test, 0.05, 5), gl.MIXED)
    _, ol, ms_l, finfo = L.solve_learned(gl, s, test, gl.MIXED)
    s.close()
    assert np.all(ob["residual"] <= 1e-10) and np.all(ol["residual"] <= 1e-10)
    assert finfo["fallbacks"] == 0
    assert ol["newton_its"].sum() < ob["newton_its"].sum(), (ol["newton_its"], ob["newton_its"])
    assert ol["gmres_its"].sum() < ob["gmres_its"].sum(), (ol["gmres_its"], ob["gmres_its"])
    assert ms_l < ms_b, (ms_l, ms_b)
    assert np.allclose(ol["free_energy"], ob["free_energy"], rtol=1e-9)
