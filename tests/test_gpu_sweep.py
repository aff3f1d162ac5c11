"""A sweep solved in waves of batched contexts gives each instance the minimum it reaches in a
single context holding the whole sweep.  The preconditioner's storage and kernel shapes follow
the context's total size (FP16 coarse levels from 2000 nodes, warps per block row), so the
FP32 Krylov path of an instance changes with its wave at rounding level: the converged free
energies agree to the Newton tolerance, not bitwise."""
import importlib

import numpy as np
import pytest

from _lib import product

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gl():
    return product()


def test_waves_match_single_context(gl):
    sweep = importlib.import_module("verkko-hem-repo_gb300.sweep")
    pts = [(20.0, 0.6, 8.0, 6), (12.0, 0.45, 12.0, 9), (30.0, 0.85, 10.0, 7), (5.0, 0.7, 9.0, 8)]
    meshes = [gl.box_mesh([-5.0, -5.0, -D / 2], [5.0, 5.0, D / 2], (n, n, n)) for _, _, D, n in pts]
    prms = [gl.Params.from_matep(p, t, precision=gl.MIXED, precond=gl.PC_MULTIGRID) for p, t, _, _ in pts]
    x0 = [gl.bphase_guess(p, t, m.nn, noise=0.05, seed=k) for k, ((p, t, _, _), m) in enumerate(zip(pts, meshes))]
    kw = dict(linear_tol=1e-4, converge_acc=1e-10)
    one = sweep.solve_sweep(gl, meshes, prms, x0, budget=1e12, **kw)
    assert one["waves"] == [4]
    nn_max = max(m.nn for m in meshes)
    per = one["bytes_per_node"]
    assert per > 1000.0 and one["wave_bytes"][0] <= 1.1 * per * sum(m.nn for m in meshes)
    many = sweep.solve_sweep(gl, meshes, prms, x0, budget=1.1 * per * nn_max * 1.05, keep_solutions=True, **kw)
    assert len(many["waves"]) >= 3 and sum(many["waves"]) == 4
    for r in (one, many):
        assert r["converged"].all() and (r["residual"] <= 1e-10).all()
    assert np.allclose(many["free_energy"], one["free_energy"], rtol=1e-10, atol=0)
    assert [s.size for s in many["solutions"]] == [18 * m.nn for m in meshes]
    with pytest.raises(ValueError):
        sweep.solve_sweep(gl, meshes, prms, x0, budget=0.5 * per * nn_max, **kw)
