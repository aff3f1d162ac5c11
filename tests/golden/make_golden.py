"""Generates the golden fixtures in this directory from the reference's own code.

Run from the repository root on a machine that has the reference tree:

    python tests/golden/make_golden.py [REFERENCE_ROOT]

It compiles the reference's cell kernels (femgl/src/cell_mat_vec/*.cc) and
material parameters (matep/src/matep.cc) unmodified with
``oracle/refshim/build_ref.sh`` and records, for fixed seeds:

* ``kernels.npz``: the 18 per-(i,j,q) kernels on random dense test/trial tensors
  and random iterates (values and gradients);
* ``matep.json``: Matep coefficients on a (p, t, SCC) grid;
* ``cell.npz``: one Q1 cell (h = 0.625, the 32^3 cube's spacing) assembled the way
  femgl/src/assemble.cc:188-280 does it, i.e. 165,888 (i,j,q) tuples each calling
  the nine reference kernels: the 144x144 cell matrix and the cell right-hand side;
* ``face.npz``: the Robin (AdGR) term of each of the six faces of one anisotropic cell,
  assembled the way femgl/src/assemble.cc:286-348 does it with the reference's face
  kernels (bt = 3);
* ``pdw.npz``: the reference's weak-coupling PDW initial state (femgl/inc/pdw_config.h)
  at 64 points of a slab, at p = 20 bar, t = 0.6.

The tests read only these files; nothing at test time needs the reference tree.
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def main(ref_root: str | None = None) -> None:
    cmd = ["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"]
    if ref_root:
        cmd.append(f"REFERENCE_ROOT={ref_root}")
    subprocess.run(cmd, check=True)
    from oracle import gl

    R = gl.ref()
    if R is None:
        raise SystemExit("reference kernels not built")
    dp = gl._dp

    def p(a):
        return np.ascontiguousarray(a, np.float64).ctypes.data_as(dp)

    rng = np.random.default_rng(20240601)
    n = 64
    A = rng.standard_normal((n, 18)) * 1.5
    Pi = rng.standard_normal((n, 18))
    Pj = rng.standard_normal((n, 18))
    gA = rng.standard_normal((n, 54))
    gPi = rng.standard_normal((n, 54))
    gPj = rng.standard_normal((n, 54))
    bulk_vec = np.array([[R.ref_bulk_vec(t, p(A[s]), p(Pi[s])) for t in range(6)] for s in range(n)])
    bulk_mat = np.array([[R.ref_bulk_mat(t, p(A[s]), p(Pi[s]), p(Pj[s])) for t in range(6)] for s in range(n)])
    grad_vec = np.array([[R.ref_grad_vec(t, p(gA[s]), p(gPi[s])) for t in range(2)] for s in range(n)])
    grad_mat = np.array([[R.ref_grad_mat(t, p(gPi[s]), p(gPj[s])) for t in range(2)] for s in range(n)])
    face_vec = np.array([R.ref_face_vec(p(A[s]), p(Pi[s])) for s in range(n)])
    face_mat = np.array([R.ref_face_mat(p(Pi[s]), p(Pj[s])) for s in range(n)])
    np.savez_compressed(os.path.join(OUT, "kernels.npz"), A=A, Pi=Pi, Pj=Pj, gA=gA, gPi=gPi, gPj=gPj,
                        bulk_vec=bulk_vec, bulk_mat=bulk_mat, grad_vec=grad_vec, grad_mat=grad_mat,
                        face_vec=face_vec, face_mat=face_mat)

    rows = []
    out = np.zeros(13)
    for scc in (1, 0):
        for pr in (0.0, 1.5, 2.0, 7.3, 13.999, 20.0, 21.22, 27.5, 33.9):
            for t in (0.3, 0.6, 0.8, 0.95, 1.0):
                R.ref_matep(pr, t, scc, out.ctypes.data_as(dp))
                rows.append({"p": pr, "t": t, "scc": scc, "out": [float(v) for v in out]})
    with open(os.path.join(OUT, "matep.json"), "w") as f:
        json.dump({"fields": ["alpha", "beta1", "beta2", "beta3", "beta4", "beta5", "gap_A", "gap_B", "Tc_mK",
                              "f_A", "f_B", "beta_A", "beta_B"], "rows": rows}, f, indent=1)

    # one cell, verbatim reference loop structure
    m20 = [r for r in rows if r["p"] == 20.0 and r["t"] == 0.6 and r["scc"] == 1][0]["out"]
    coef9 = np.array([gl.K_REF, gl.K_REF, gl.K_REF, m20[0], *m20[1:6]])
    h = np.array([0.625, 0.625, 0.625])
    gapB = m20[7]
    x = np.zeros((8, 18))
    x[:, 0] = x[:, 4] = x[:, 8] = gapB * np.float32(0.577350269)
    x += 0.3 * rng.standard_normal((8, 18))
    K = np.zeros(144 * 144)
    r = np.zeros(144)
    R.ref_cell_assemble(p(h), p(x), p(coef9), K.ctypes.data_as(dp), r.ctypes.data_as(dp))
    np.savez_compressed(os.path.join(OUT, "cell.npz"), h=h, x=x, coef9=coef9, cell_matrix=K.reshape(144, 144),
                        cell_rhs=r)

    # the Robin faces of one anisotropic cell, verbatim reference face loop (assemble.cc:286-348)
    frng = np.random.default_rng(20240602)
    hf = np.array([0.5, 0.625, 0.75])
    xf = frng.standard_normal((8, 18))
    bt = 3.0
    Kf = np.zeros((6, 144 * 144))
    rf = np.zeros((6, 144))
    for face in range(6):
        R.ref_face_assemble(p(hf), p(xf), ctypes.c_double(gl.K_REF), ctypes.c_double(bt), face,
                            Kf[face].ctypes.data_as(dp), rf[face].ctypes.data_as(dp))
    np.savez_compressed(os.path.join(OUT, "face.npz"), h=hf, x=xf, K1=gl.K_REF, bt=bt,
                        face_matrix=Kf.reshape(6, 144, 144), face_rhs=rf)

    # the weak-coupling PDW initial state (femgl/inc/pdw_config.h) at random points of a slab,
    # with the parameters setup_weak-coupling-PDW-configuration.cc:286-315 passes
    prng = np.random.default_rng(20240603)
    half_D, u_amp = 5.0, 0.3
    q = 3.141592653589793 / (1.7320508075688772 * 2.0 * half_D)
    pts = np.column_stack([prng.uniform(-12, 12, 64), prng.uniform(-12, 12, 64), prng.uniform(-half_D, half_D, 64)])
    pts[:4, 2] = [-half_D, half_D, 0.0, -half_D]
    vals = np.zeros((64, 18))
    for i in range(64):
        R.ref_pdw_value(u_amp, q, half_D, gapB, *pts[i], vals[i].ctypes.data_as(dp))
    np.savez_compressed(os.path.join(OUT, "pdw.npz"), p=20.0, t=0.6, scc=1, u=u_amp, half_D=half_D, gap=gapB,
                        points=pts, values=vals)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
