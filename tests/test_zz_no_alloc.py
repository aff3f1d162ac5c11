"""GPU test of glgpu_dot_noalloc, the entry point that allocates nothing.

It serves callers that cannot call cudaMalloc where they need a norm (inside stream
capture, allocation-free loops, or host frameworks that own all device memory): they
pass their own device vectors and a device output, and the reduction's partial sums
live in a fixed array inside the library.  This test plays such a caller: it owns the
device buffers (allocated here through the CUDA runtime), calls the entry point twice
in a row through the C ABI, and checks each result against the existing entry point
glgpu_compute_residual, whose norm comes from the context's own reduction.
"""
import ctypes
import math

import numpy as np
import pytest

from _lib import product

pytestmark = pytest.mark.gpu

MAX_N = 16384 * 1024


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            rt = None
    if rt is None:
        pytest.skip("CUDA runtime library not found")
    rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaFree.argtypes = [ctypes.c_void_p]
    return rt


H2D, D2H = 1, 2


def test_dot_noalloc_matches_context_norm_twice():
    gl = product()
    L = gl.lib()
    rt = _cudart()
    m = gl.cube_mesh(2.5, 4, 0.25)
    prm = gl.Params.from_matep(20.0, 0.6)
    starts = [gl.bphase_guess(20.0, 0.6, m.nn, noise=0.1, seed=s) for s in (1, 2)]
    n = 18 * m.nn
    d_vec, d_out = ctypes.c_void_p(), ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(d_vec), 8 * n) == 0
    assert rt.cudaMalloc(ctypes.byref(d_out), 8) == 0
    try:
        with gl.FemGL(m, prm) as f:
            for x0 in starts:  # two calls in a row, different data
                f.set_solution(x0)
                norm_ctx = float(f.compute_residual()[0])
                R = np.ascontiguousarray(f.residual())
                assert rt.cudaMemcpy(d_vec, R.ctypes.data, 8 * n, H2D) == 0
                st = L.glgpu_dot_noalloc(d_vec, d_vec, n, d_out, None)
                assert st == 0, L.glgpu_last_error().decode()
                out = np.zeros(1)
                assert rt.cudaMemcpy(out.ctypes.data, d_out, 8, D2H) == 0
                assert abs(math.sqrt(out[0]) - norm_ctx) <= 1e-12 * norm_ctx
        # sizes beyond the fixed scratch are rejected before any work is enqueued
        assert L.glgpu_dot_noalloc(d_vec, d_vec, MAX_N + 1, d_out, None) == 1
        assert b"exceeds the maximum" in L.glgpu_last_error()
    finally:
        rt.cudaFree(d_vec)
        rt.cudaFree(d_out)


@pytest.mark.parametrize("n", [0, 1_000_003, MAX_N])
def test_dot_noalloc_sizes_against_host_dot(n):
    """Lengths the first test does not reach: none, a large ragged last segment (more
    than 256 partials, so each lane of the final pass sums several) and the maximum.
    Checked against an exactly rounded host sum, within 1e-12 of sum |x_i y_i|, and
    bitwise equal over two calls on the same data (the reduction order is fixed)."""
    gl = product()
    L = gl.lib()
    rt = _cudart()
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    y = rng.standard_normal(n)
    d_x, d_y, d_out = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(d_x), max(8, 8 * n)) == 0
    assert rt.cudaMalloc(ctypes.byref(d_y), max(8, 8 * n)) == 0
    assert rt.cudaMalloc(ctypes.byref(d_out), 8) == 0
    try:
        if n:
            assert rt.cudaMemcpy(d_x, x.ctypes.data, 8 * n, H2D) == 0
            assert rt.cudaMemcpy(d_y, y.ctypes.data, 8 * n, H2D) == 0
        got = []
        for _ in range(2):
            st = L.glgpu_dot_noalloc(d_x, d_y, n, d_out, None)
            assert st == 0, L.glgpu_last_error().decode()
            out = np.zeros(1)
            assert rt.cudaMemcpy(out.ctypes.data, d_out, 8, D2H) == 0
            got.append(out[0])
        exact = math.fsum((x * y).tolist()) if n else 0.0
        scale = float(np.abs(x * y).sum()) if n else 0.0
        assert abs(got[0] - exact) <= 1e-12 * scale, (got[0], exact)
        assert got[0] == got[1]
        if n == 0:
            assert got[0] == 0.0
    finally:
        rt.cudaFree(d_x)
        rt.cudaFree(d_y)
        rt.cudaFree(d_out)
