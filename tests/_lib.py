"""Test helpers: import the product package (its directory name has hyphens)."""
import importlib
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def product():
    pkg = importlib.import_module("verkko-hem-repo_gb300")
    pkg.build()
    return pkg


def coef_of(params):
    """Oracle coefficient vector {K1, K2+K3, alpha, beta1..5, K1/bt} of a product Params."""
    import numpy as np

    wR = params.K1 / params.bt if params.bt < 1e10 else 0.0
    return np.array([params.K1, params.K2 + params.K3, params.alpha, *params.beta, wR], dtype=np.float64)


def oracle_mesh(m):
    """Product Mesh -> oracle Mesh (same arrays)."""
    from oracle import mesh as om
    import numpy as np

    hptr = m.hptr if m.hptr is not None else np.zeros(m.nn + 1, np.int32)
    hpar = m.hpar if m.hpar is not None else np.zeros(0, np.int32)
    hw = m.hw if m.hw is not None else np.zeros(0)
    return om.Mesh(xyz=m.xyz, cells=m.cells, mask=m.mask, hptr=hptr, hpar=hpar, hw=hw)
