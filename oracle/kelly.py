"""Kelly error estimator, FP64 CPU restatement (TEST INFRASTRUCTURE: the checker of the GPU
estimator, never part of the product).

deal.II's KellyErrorEstimator::estimate as the reference calls it (femgl/src/refine.cc:147-152:
QGauss<2>(2) on faces, no Neumann boundary map, all components, the default strategy):

    eta_K = sqrt( h_K / 24 * sum over faces F of K of int_F |[du/dn]|^2 dS ),   h_K = diameter,

boundary faces contributing nothing, faces of periodic pairs counting as interior, and on a
face between a coarse and four fine cells the integral taken over each fine face (it counts
for the fine cell and for the coarse cell).  refine_and_coarsen_fixed_number then flags the
floor(top * n) cells of largest eta (every cell >= that rank's value).

Neighbours are found here by point location on the mesher's half-cell lattice (a point half a
lattice unit outside each face quadrature point), not from node keys as the product does.
"""
from __future__ import annotations

import numpy as np

G = 0.5 - np.sqrt(3.0) / 6.0


def kelly(m, x, lo, hi, n, periodic=(False, False), return_pairs=False):
    """eta per cell; with return_pairs also the set of face pairs (a, face of a, b, sub):
    sub = 1 for a fine face a inside the face of coarse cell b, 0 for coinciding faces
    (listed once, a < b)."""
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    n = np.asarray(n, int)
    hf = (hi - lo) / n / 2.0  # lattice unit: half a cell of the n-grid
    X = np.asarray(x, float).reshape(-1, 18)
    x0 = m.xyz[m.cells[:, 0]]
    x7 = m.xyz[m.cells[:, 7]]
    corner = np.rint((x0 - lo) / hf).astype(int)
    size = np.rint((x7[:, 0] - x0[:, 0]) / hf[0]).astype(int)
    where = {(tuple(c), int(s)): e for e, (c, s) in enumerate(zip(corner, size))}
    ext = 2 * n

    def locate(p):
        p = p.copy()
        for a in range(2):
            if periodic[a]:
                p[a] = p[a] % ext[a]
        if np.any(p < 0) or np.any(p > ext):
            return None, None
        f = np.floor(p).astype(int)
        e = where.get((tuple(f), 1))
        if e is not None:
            return e, p
        c = 2 * np.floor(p / 2).astype(int)
        return where.get((tuple(c), 2)), p

    def dn(e, ax, p):
        # normal derivative of the Q1 field of cell e at lattice point p
        s = size[e]
        xi = (p - corner[e]) / s
        out = np.zeros(18)
        for v in range(8):
            w = 1.0 / (s * hf[ax]) * (1 if (v >> ax) & 1 else -1)
            for t in range(3):
                if t != ax:
                    w *= xi[t] if (v >> t) & 1 else 1.0 - xi[t]
            out += w * X[m.cells[e, v]]
        return out

    eta2 = np.zeros(m.nc)
    pairs = set()
    for e in range(m.nc):
        s = size[e]
        for f in range(6):
            ax, side = divmod(f, 2)
            t1, t2 = [t for t in range(3) if t != ax]
            area = (s * hf[t1]) * (s * hf[t2])
            nbs = []
            acc = 0.0
            for q1 in (G, 1 - G):
                for q2 in (G, 1 - G):
                    p = corner[e].astype(float)
                    p[ax] += side * s
                    p[t1] += q1 * s
                    p[t2] += q2 * s
                    out = p.copy()
                    out[ax] += 0.5 if side else -0.5
                    b, pb = locate(out)
                    nbs.append(b)
                    if b is None:
                        continue
                    pb = pb.copy()
                    pb[ax] -= 0.5 if side else -0.5
                    j = dn(e, ax, p) - dn(b, ax, pb)
                    acc += (area / 4.0) * float(j @ j)
            if any(b is None for b in nbs):
                assert all(b is None for b in nbs)
                continue  # boundary face
            nb = nbs[0]
            if size[nb] > s:  # coarse neighbour: this fine face counts for both
                eta2[e] += acc
                eta2[nb] += acc
                pairs.add((e, f, nb, 1))
            elif size[nb] == s:
                eta2[e] += acc
                pairs.add((min(e, nb), f if e < nb else f ^ 1, max(e, nb), 0))
            # a finer neighbour adds this cell's share from its own side
    h = (x7 - x0)
    diam = np.sqrt((h * h).sum(axis=1))
    if return_pairs:
        return np.sqrt(eta2 * diam / 24.0), pairs
    return np.sqrt(eta2 * diam / 24.0)


def fixed_number_flags(eta, top, bottom=0.0):
    """deal.II GridRefinement::refine_and_coarsen_fixed_number on one triangulation."""
    eta = np.asarray(eta)
    nk = eta.size
    kr, kc = int(top * nk), int(bottom * nk)
    flags = np.zeros(nk, np.int8)
    if kr > 0:
        thr = np.sort(eta)[::-1][kr - 1]
        flags[eta >= thr] = 1
    if kc > 0:
        thr = np.sort(eta)[kc - 1]
        flags[(eta <= thr) & (flags == 0)] = -1
    return flags
