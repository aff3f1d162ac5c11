"""Python side of the oracle (TEST INFRASTRUCTURE ONLY).

Loads the oracle's C restatement (``oracle/_build/libgloracle.so``, built from
``oracle/gl_oracle.c``) and, when present, the reference's own kernels compiled
unmodified (``oracle/_ref/libglref.so``, built by ``oracle/refshim/build_ref.sh``).

Also restates the reference's damped Newton loop:

* ``newton_iteration`` (reference femgl/src/iteration.cc:130-210): previous
  residual = ||system_rhs||; for i < 100: a = step**i, x_trial = x + a*delta,
  constraints distribute, residual at x_trial, accept on the first strict
  decrease; when no trial decreases the residual the last trial is kept;
* ``run`` (femgl/src/run.cc:207-256): assemble, solve, newton_iteration, stop when
  ||R|| <= converge accuracy;
* ``solve`` (femgl/src/solve.cc:159-183): J delta = rhs, delta distributed through
  the constraints.  The oracle solves the unconstrained block exactly (sparse LU)
  instead of FGMRES+AMG, so that Newton counts do not depend on a preconditioner.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from . import mesh as omesh

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libgloracle.so")
REF_SO = os.path.join(HERE, "_ref", "libglref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_up = ctypes.POINTER(ctypes.c_uint32)


def build(quiet: bool = True) -> None:
    """Compile the oracle restatement (and the reference kernels when the
    reference tree is present)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE, "all", "ref"], check=True, stdout=out)


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        L.orc_bulk_q.argtypes = [_dp, _dp, _dp, _dp, _dp]
        L.orc_cell_local.argtypes = [_dp, _dp, _dp, ctypes.c_int, _dp, _dp, _dp]
        L.orc_pattern.restype = ctypes.c_long
        L.orc_pattern.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _ip, _ip, _dp, _ip, _ip]
        L.orc_assemble.restype = ctypes.c_int
        L.orc_assemble.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _up, _ip, _ip, _dp, _dp, _dp, _ip, _ip,
                                   _dp, _dp, _dp]
        L.orc_distribute.argtypes = [ctypes.c_int, _up, _ip, _ip, _dp, _dp]
        L.orc_robin_faces.argtypes = [ctypes.c_int, _ip, _up, _ip, _ip, ctypes.POINTER(ctypes.c_uint8)]
        L.orc_spmv.argtypes = [ctypes.c_int, _ip, _ip, _dp, _dp, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_gmres.restype = ctypes.c_int
        L.orc_gmres.argtypes = [ctypes.c_int, _ip, _ip, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp,
                                _dp]
        L.orc_bphase_guess.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_uint64, _dp]
        _lib = L
    return _lib


def ref():
    """The reference's own kernels, or None when they were not built here."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        L = ctypes.CDLL(REF_SO)
        for f in ("ref_bulk_mat", "ref_bulk_vec", "ref_grad_mat", "ref_grad_vec", "ref_face_mat", "ref_face_vec"):
            getattr(L, f).restype = ctypes.c_double
        L.ref_bulk_mat.argtypes = [ctypes.c_int, _dp, _dp, _dp]
        L.ref_bulk_vec.argtypes = [ctypes.c_int, _dp, _dp]
        L.ref_grad_mat.argtypes = [ctypes.c_int, _dp, _dp]
        L.ref_grad_vec.argtypes = [ctypes.c_int, _dp, _dp]
        L.ref_matep.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp]
        L.ref_cell_assemble.argtypes = [_dp, _dp, _dp, _dp, _dp]
        L.ref_face_assemble.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp]
        L.ref_pdw_value.argtypes = [ctypes.c_double] * 7 + [_dp]
        _ref = L
    return _ref


# ---------------------------------------------------------------------------------
# coefficients
# ---------------------------------------------------------------------------------
K_REF = 0.42072  # K1 = K2 = K3 (reference femgl/inc/femgl.h:320-322)


def coef_vector(alpha, betas, K1=K_REF, K2=K_REF, K3=K_REF, bt=1e10):
    """{K1, K2+K3, alpha, beta1..beta5, K1/bt}: the weights of assemble.cc:229-252 and of
    the Robin faces (assemble.cc:286-348; 0 when bt >= 1e10)."""
    return np.array([K1, K2 + K3, alpha, *betas, K1 / bt if bt < 1e10 else 0.0], dtype=np.float64)


def _coef9(coef):
    c = np.zeros(9)
    c[: len(coef)] = coef
    return c


MATEP_FIELDS = ("alpha", "beta1", "beta2", "beta3", "beta4", "beta5", "gap_A", "gap_B", "Tc_mK", "f_A", "f_B",
                "beta_A", "beta_B")
GOLDEN_MATEP = os.path.join(os.path.dirname(HERE), "tests", "golden", "matep.json")


def matep(p: float, t: float, scc: bool = True) -> dict:
    """The reference's material parameters at (p bar, t = T/Tc): from its own matep
    (matep/src/matep.cc, compiled unmodified into oracle/_ref) where that was built, else
    from the committed table of that compiled matep's outputs (tests/golden/matep.json,
    90 (p, t, SCC) points).  Raises KeyError for a point the table lacks."""
    R = ref()
    if R is not None:
        out = np.zeros(13)
        R.ref_matep(float(p), float(t), int(bool(scc)), _p(out))
        return dict(zip(MATEP_FIELDS, out.tolist()))
    import json

    with open(GOLDEN_MATEP) as fh:
        rows = json.load(fh)["rows"]
    for r in rows:
        if r["p"] == float(p) and r["t"] == float(t) and r["scc"] == int(bool(scc)):
            return dict(zip(MATEP_FIELDS, r["out"]))
    raise KeyError(f"matep({p}, {t}, scc={scc}) is not in the golden table and oracle/_ref is not built")


def bphase_guess(gap_B: float, nn: int, noise: float = 0.0, seed: int = 0) -> np.ndarray:
    """Uniform B-phase start (setup_uniform_B-phase.cc:238-259) plus the configurations'
    seeded noise; not yet distributed through the constraints."""
    x = np.zeros(18 * int(nn))
    lib().orc_bphase_guess(float(gap_B), int(nn), float(noise), int(seed), _p(x))
    return x


def time_reference_cells(h, x_cells, coef9, threads: int = 1):
    """Times the reference's own Jacobian + rhs loop over one Q1 cell at a time
    (femgl/src/assemble.cc:188-280: q x i x j with the 18 cell_mat_vec kernels, compiled
    unmodified into oracle/_ref) on the cell states x_cells [n][8][18], spread over
    `threads` host threads.  coef9 = (K1, K2, K3, alpha, beta1..beta5).  Returns (seconds
    of wall time, the cell matrices [n][144][144], the cell rhs [n][144]).  Needs oracle/_ref."""
    import time
    from concurrent.futures import ThreadPoolExecutor

    R = ref()
    if R is None:
        raise RuntimeError("oracle/_ref (the reference's kernels) is not built on this host")
    h = np.ascontiguousarray(h, np.float64)
    c9 = np.ascontiguousarray(coef9, np.float64)
    xs = np.ascontiguousarray(x_cells, np.float64).reshape(-1, 144)
    n = xs.shape[0]
    K = np.zeros((n, 144, 144))
    r = np.zeros((n, 144))

    def one(k):
        R.ref_cell_assemble(_p(h), _p(xs[k]), _p(c9), _p(K[k]), _p(r[k]))

    t0 = time.perf_counter()
    if threads <= 1:
        for k in range(n):
            one(k)
    else:  # ctypes releases the interpreter lock for the duration of each call
        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(one, range(n)))
    return time.perf_counter() - t0, K, r


def gauge_align(x, ref, iters: int = 20):
    """x moved onto ref by the exact symmetries of the functional: a global phase
    e^{i phi} and a spin rotation R (A -> e^{i phi} R A, acting on the spin index mu of
    A_{mu j}; the zero-Dirichlet columns stay zero).  The free energy and the residual norm
    are invariant, and so is the solution set: near a minimum the Jacobian is singular
    along these directions, so Newton runs that differ only in their linear solves stop at
    different points of the same orbit.  (phi, R) maximise Re tr(e^{i phi} R C), C = sum
    over nodes of A B^+ (B the reference), by alternating the phase and the orthogonal
    Procrustes rotation.  Returns (aligned x, phi, R)."""
    X = np.asarray(x, np.float64).reshape(-1, 18)
    Y = np.asarray(ref, np.float64).reshape(-1, 18)
    A = (X[:, :9] + 1j * X[:, 9:]).reshape(-1, 3, 3)
    B = (Y[:, :9] + 1j * Y[:, 9:]).reshape(-1, 3, 3)
    C = np.einsum("nij,nkj->ik", A, B.conj())  # sum_n A_n B_n^+
    R = np.eye(3)
    phi = 0.0
    for _ in range(iters):
        phi = -float(np.angle(np.trace(R @ C)))
        M = np.real(np.exp(1j * phi) * C)  # maximise tr(R M)
        U, _, Vt = np.linalg.svd(M)
        D = np.diag([1.0, 1.0, np.sign(np.linalg.det(Vt.T @ U.T))])
        R = Vt.T @ D @ U.T
    Al = np.exp(1j * phi) * np.einsum("ij,njk->nik", R, A)
    out = np.concatenate([Al.real.reshape(-1, 9), Al.imag.reshape(-1, 9)], axis=1).reshape(-1)
    return out, phi, R


# ---------------------------------------------------------------------------------
# per-q and per-cell physics
# ---------------------------------------------------------------------------------
def bulk_q(coef, A):
    R = np.zeros(18)
    H = np.zeros(324)
    f = np.zeros(1)
    lib().orc_bulk_q(_p(_coef9(coef)), _p(np.ascontiguousarray(A, np.float64)), _p(R),
                     _p(H), _p(f))
    return R, H.reshape(18, 18), float(f[0])


def cell_local(h, x, coef, want_K=True, faces=0):
    """One cell's matrix, residual pieces and energy; faces: bitmask of its Robin faces."""
    h = np.ascontiguousarray(h, np.float64)
    x = np.ascontiguousarray(x, np.float64).reshape(144)
    K = np.zeros((144, 144)) if want_K else None
    r = np.zeros(144)
    f = np.zeros(1)
    lib().orc_cell_local(_p(h), _p(x), _p(_coef9(coef)), int(faces), _p(K) if want_K else None, _p(r), _p(f))
    return K, r, float(f[0])


# ---------------------------------------------------------------------------------
# mesh-level system
# ---------------------------------------------------------------------------------
class System:
    """Condensed FP64 system on one mesh (femgl 3D, 18 components)."""

    def __init__(self, m: omesh.Mesh, coef):
        self.m = m
        self.coef = _coef9(coef)
        self.xyz = np.ascontiguousarray(m.xyz, np.float64)
        self.cells = np.ascontiguousarray(m.cells, np.int32)
        self.mask = np.ascontiguousarray(m.mask, np.uint32)
        self.hptr = np.ascontiguousarray(m.hptr, np.int32)
        self.hpar = np.ascontiguousarray(m.hpar, np.int32)
        self.hw = np.ascontiguousarray(m.hw, np.float64)
        L = lib()
        nnzb = L.orc_pattern(m.nn, m.nc, _p(self.cells, _ip), _p(self.hptr, _ip), _p(self.hpar, _ip), _p(self.hw),
                             None, None)
        self.rowptr = np.zeros(m.nn + 1, dtype=np.int32)
        self.cols = np.zeros(nnzb, dtype=np.int32)
        L.orc_pattern(m.nn, m.nc, _p(self.cells, _ip), _p(self.hptr, _ip), _p(self.hpar, _ip), _p(self.hw),
                      _p(self.rowptr, _ip), _p(self.cols, _ip))
        self.nnzb = int(nnzb)
        self.nd = 18 * m.nn
        free = np.ones((m.nn, 18), dtype=bool)
        hanging = np.diff(self.hptr) > 0
        free[hanging, :] = False
        for c in range(18):
            free[(self.mask >> np.uint32(c)) & np.uint32(1) == 1, c] = False
        free[hanging, :] = False
        self.free = free.ravel()

    def robin_faces(self):
        """Per cell the bits f = 2 axis + side of its Robin (pair-breaking) faces."""
        out = np.zeros(self.m.nc, np.uint8)
        lib().orc_robin_faces(self.m.nc, _p(self.cells, _ip), _p(self.mask, _up), _p(self.hptr, _ip),
                              _p(self.hpar, _ip), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        return out

    def assemble(self, x, want_J=True):
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        J = np.zeros(self.nnzb * 324) if want_J else None
        R = np.zeros(self.nd)
        F = np.zeros(1)
        err = lib().orc_assemble(self.m.nn, _p(self.xyz), self.m.nc, _p(self.cells, _ip), _p(self.mask, _up),
                                 _p(self.hptr, _ip), _p(self.hpar, _ip), _p(self.hw), _p(self.coef), _p(x),
                                 _p(self.rowptr, _ip), _p(self.cols, _ip), _p(J) if want_J else None, _p(R), _p(F))
        if err != 0:
            raise RuntimeError("oracle assembly: block outside the pattern")
        return (J.reshape(self.nnzb, 18, 18) if want_J else None), R, float(F[0])

    def residual(self, x):
        _, R, F = self.assemble(x, want_J=False)
        return R, F

    def distribute(self, x):
        x = np.array(x, dtype=np.float64).reshape(-1)
        lib().orc_distribute(self.m.nn, _p(self.mask, _up), _p(self.hptr, _ip), _p(self.hpar, _ip), _p(self.hw),
                             _p(x))
        return x

    def spmv(self, J, x):
        y = np.zeros(self.nd)
        lib().orc_spmv(self.m.nn, _p(self.rowptr, _ip), _p(self.cols, _ip),
                       _p(np.ascontiguousarray(J, np.float64).reshape(-1)), _p(np.ascontiguousarray(x, np.float64)),
                       _p(y))
        return y

    def to_scipy(self, J):
        import scipy.sparse as sp
        nn = self.m.nn
        rows = np.repeat(np.arange(nn), np.diff(self.rowptr))
        bsr = sp.bsr_matrix((np.asarray(J).reshape(-1, 18, 18), self.cols, self.rowptr), shape=(18 * nn, 18 * nn))
        return bsr.tocsr(), rows

    def block_of(self, J, row, col):
        k0, k1 = self.rowptr[row], self.rowptr[row + 1]
        idx = np.searchsorted(self.cols[k0:k1], col)
        if idx >= k1 - k0 or self.cols[k0 + idx] != col:
            return None
        return J[k0 + idx]

    def solve_gmres(self, J, rhs, tol=1e-10, restart=50, max_it=10000):
        """Block-Jacobi GMRES(restart) on all host threads (the timed CPU baseline's
        linear solve).  Returns (delta distributed, iterations, relative residual)."""
        d = np.zeros(self.nd)
        rel = np.zeros(1)
        its = lib().orc_gmres(self.m.nn, _p(self.rowptr, _ip), _p(self.cols, _ip),
                              _p(np.ascontiguousarray(J, np.float64).reshape(-1)),
                              _p(np.ascontiguousarray(rhs, np.float64)), float(tol), int(restart), int(max_it), _p(d),
                              _p(rel))
        return self.distribute(d), int(its), float(rel[0])

    def solve_exact(self, J, rhs):
        """delta with J_ff delta_f = rhs_f on the unconstrained dofs (sparse LU), then
        distributed through the constraints (reference femgl/src/solve.cc:181)."""
        import scipy.sparse.linalg as spla
        A, _ = self.to_scipy(J)
        f = np.flatnonzero(self.free)
        Aff = A[f][:, f].tocsc()
        d = np.zeros(self.nd)
        d[f] = spla.spsolve(Aff, rhs[f])
        return self.distribute(d)


def newton(system, x0, tol=1e-10, max_iter=40, step=0.83, max_trials=100, damped=True, log=None,
           linear_tol=None, restart=50):
    """The reference's outer loop (run.cc:207-256) with its damped Newton step
    (iteration.cc:130-210).  The linear solve is exact (sparse LU) by default, or
    block-Jacobi GMRES(restart) to linear_tol * ||rhs|| (solve.cc:159-160) when
    linear_tol is given.  Returns (x, history) with one dict per Newton iteration."""
    x = system.distribute(x0)
    hist = []
    for it in range(max_iter + 1):
        J, R, F = system.assemble(x)
        rhs = -R
        prev = float(np.linalg.norm(rhs))
        lin_its = 0
        if linear_tol is None:
            delta = system.solve_exact(J, rhs)
        else:
            delta, lin_its, _ = system.solve_gmres(J, rhs, tol=linear_tol, restart=restart)
        trials = 0
        x_trial = x
        cur = None
        n_trials = max_trials if damped else 1
        for i in range(n_trials):
            a = step ** i if damped else 1.0
            x_trial = system.distribute(x + a * delta)
            Rt, Ft = system.residual(x_trial)
            cur = float(np.linalg.norm(Rt))
            trials = i + 1
            if cur < prev:
                break
        x = x_trial
        hist.append({"iter": it, "res_before": prev, "res": cur, "trials": trials, "F": Ft, "linear_its": lin_its})
        if log:
            log(hist[-1])
        if cur <= tol:
            break
    return x, hist


# ---------------------------------------------------------------------------------
# complexGL 2D (config 1) restated in numpy from the reference's archive solver
# complexGL-src-archive/complexGL.cc:479-548 (gradient weight 1/2, bulk alpha + beta|psi|^2)
# ---------------------------------------------------------------------------------
class System2D:
    def __init__(self, m: omesh.Mesh2D, alpha=-1.0, beta=0.5, K=1.0):
        self.m = m
        self.alpha, self.beta, self.K = float(alpha), float(beta), float(K)
        n = m.nn
        self.nd = 2 * n
        h = m.xy[m.cells[0, 3]] - m.xy[m.cells[0, 0]]
        self.h = h
        g = 0.5 - np.sqrt(3.0) / 6.0
        gp = np.array([g, 1 - g])
        val = np.zeros((4, 4))
        grd = np.zeros((4, 4, 2))
        for q in range(4):
            xi = np.array([gp[q & 1], gp[(q >> 1) & 1]])
            for v in range(4):
                b = np.array([(v >> 0) & 1, (v >> 1) & 1])
                s = np.where(b == 1, xi, 1 - xi)
                ds = np.where(b == 1, 1.0, -1.0) / h
                val[q, v] = s[0] * s[1]
                grd[q, v] = [ds[0] * s[1], s[0] * ds[1]]
        self.val, self.grd = val, grd
        self.JxW = 0.25 * h[0] * h[1]
        free = np.ones((n, 2), dtype=bool)
        for c in range(2):
            free[(m.mask >> np.uint32(c)) & np.uint32(1) == 1, c] = False
        self.free = free.ravel()

    def distribute(self, x):
        x = np.array(x, dtype=np.float64).reshape(-1)
        x[~self.free] = 0.0
        return x

    def assemble(self, x, want_J=True):
        import scipy.sparse as sp
        m = self.m
        X = x.reshape(-1, 2)[m.cells]  # (nc, 4, 2)
        val, grd, JxW = self.val, self.grd, self.JxW
        r = np.zeros((m.cells.shape[0], 4, 2))
        F = 0.0
        Kloc = np.zeros((m.cells.shape[0], 8, 8)) if want_J else None
        gw = 0.5 * self.K
        for q in range(4):
            u = X[:, :, 0] @ val[q]
            v = X[:, :, 1] @ val[q]
            gu = np.einsum("cv,vk->ck", X[:, :, 0], grd[q])
            gv = np.einsum("cv,vk->ck", X[:, :, 1], grd[q])
            s2 = u * u + v * v
            bulk = self.alpha + self.beta * s2
            F += JxW * np.sum(gw * (np.sum(gu * gu, 1) + np.sum(gv * gv, 1)) + self.alpha * s2
                              + 0.5 * self.beta * s2 * s2)
            r[:, :, 0] += JxW * (gw * gu @ grd[q].T + (bulk * u)[:, None] * val[q][None, :])
            r[:, :, 1] += JxW * (gw * gv @ grd[q].T + (bulk * v)[:, None] * val[q][None, :])
            if want_J:
                GG = grd[q] @ grd[q].T
                VV = np.outer(val[q], val[q])
                huu = self.alpha + self.beta * (3 * u * u + v * v)
                hvv = self.alpha + self.beta * (3 * v * v + u * u)
                huv = 2 * self.beta * u * v
                for a in range(4):
                    for b in range(4):
                        Kloc[:, 2 * a, 2 * b] += JxW * (gw * GG[a, b] + huu * VV[a, b])
                        Kloc[:, 2 * a + 1, 2 * b + 1] += JxW * (gw * GG[a, b] + hvv * VV[a, b])
                        Kloc[:, 2 * a, 2 * b + 1] += JxW * huv * VV[a, b]
                        Kloc[:, 2 * a + 1, 2 * b] += JxW * huv * VV[a, b]
        dof = (2 * m.cells[:, :, None] + np.arange(2)[None, None, :]).reshape(-1, 8)
        R = np.zeros(self.nd)
        np.add.at(R, dof.ravel(), r.reshape(-1))
        R[~self.free] = 0.0
        J = None
        if want_J:
            rows = np.repeat(dof, 8, axis=1).ravel()
            cols = np.tile(dof, (1, 8)).ravel()
            J = sp.csr_matrix((Kloc.ravel(), (rows, cols)), shape=(self.nd, self.nd))
        return J, R, F

    def residual(self, x):
        _, R, F = self.assemble(x, want_J=False)
        return R, F

    def solve_gmres(self, J, rhs, tol=1e-10, restart=50, max_it=10000):
        """Block-Jacobi GMRES(restart) on all host threads (the timed CPU baseline's
        linear solve).  Returns (delta distributed, iterations, relative residual)."""
        d = np.zeros(self.nd)
        rel = np.zeros(1)
        its = lib().orc_gmres(self.m.nn, _p(self.rowptr, _ip), _p(self.cols, _ip),
                              _p(np.ascontiguousarray(J, np.float64).reshape(-1)),
                              _p(np.ascontiguousarray(rhs, np.float64)), float(tol), int(restart), int(max_it), _p(d),
                              _p(rel))
        return self.distribute(d), int(its), float(rel[0])

    def solve_exact(self, J, rhs):
        import scipy.sparse.linalg as spla
        f = np.flatnonzero(self.free)
        d = np.zeros(self.nd)
        d[f] = spla.spsolve(J[f][:, f].tocsc(), rhs[f])
        return d
