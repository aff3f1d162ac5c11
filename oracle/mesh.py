"""Independent numpy mesher for the oracle (TEST INFRASTRUCTURE ONLY).

Restates, for axis-aligned boxes, what the reference builds with deal.II:

* ``GridGenerator::hyper_cube`` / ``hyper_rectangle`` + ``refine_global``
  (reference femgl/src/makegrid_cube-z-normal_AdGR.cc:157-161): a tensor grid of
  Q1 hexahedra;
* boundary ids by face centre (makegrid_cube-z-normal_AdGR.cc:170-195): x/y faces
  id 1 (natural), z faces id 4;
* zero-Dirichlet component masks per boundary id
  (femgl/src/setup_uniform_B-phase.cc:139-157 with the masks of
  femgl/inc/femgl.h:294-301): id 4 (z normal) constrains components
  {2,5,8,11,14,17}, the orbital z column of u and v;
* one level of local refinement and the Q1 hanging-node constraints of
  ``DoFTools::make_hanging_node_constraints`` (setup_uniform_B-phase.cc:137):
  a fine node on a coarse edge = 1/2 of the edge's two ends, on a coarse face
  centre = 1/4 of the face's four corners.

Node numbering (shared with the CUDA library's host mesher, so arrays compare
directly): nodes are sorted by integer lattice coordinate (z, then y, then x) on
the finest lattice; cells by the lattice coordinate of their first vertex
(z, y, x) with children of a refined cell taking their own corner coordinate.
deal.II's own numbering (cell-traversal order) is not reproducible without
deal.II, so everything downstream is keyed by node coordinates.
"""
from __future__ import annotations

import dataclasses

import numpy as np

#: Dirichlet mask of boundary id 2/3/4 (x/y/z normal): orbital column 0/1/2 of u and v.
COLUMN_MASK = [sum(1 << (9 * part + 3 * mu + col) for part in range(2) for mu in range(3)) for col in range(3)]


@dataclasses.dataclass
class Mesh:
    xyz: np.ndarray  # (nn, 3) float64
    cells: np.ndarray  # (nc, 8) int32, deal.II vertex order v = ix + 2 iy + 4 iz
    mask: np.ndarray  # (nn,) uint32, bit c: component c is zero-Dirichlet
    hptr: np.ndarray  # (nn+1,) int32 hanging-constraint CSR
    hpar: np.ndarray  # int32 parents
    hw: np.ndarray  # float64 weights

    @property
    def nn(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def nc(self) -> int:
        return int(self.cells.shape[0])

    @property
    def n_hanging(self) -> int:
        return int(np.count_nonzero(np.diff(self.hptr)))


def box_mesh(lo, hi, n, refine_band: float = 0.0, dirichlet_z: bool = True, dirichlet_x: bool = False,
             dirichlet_y: bool = False, periodic_x: bool = False, periodic_y: bool = False, refine_cells=None) -> Mesh:
    """Box [lo, hi] with n = (nx, ny, nz) cells; cells whose centre lies within
    ``refine_band`` of a z face are refined once.  Zero-Dirichlet masks on the z
    faces (and optionally x, y faces) as in the reference's pair-breaking setup.
    refine_cells (flags per cell of the n-grid, x fastest) replaces the band rule.
    periodic_x / periodic_y identify the upper x / y face with the lower one
    (makegrid_retangle-z-AdGR_xy-periodic.cc:150-200; the constraints of
    DoFTools::make_periodicity_constraints, closed like AffineConstraints::close)."""
    if (dirichlet_x and periodic_x) or (dirichlet_y and periodic_y):
        raise ValueError("an axis is either pair-breaking or periodic")
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    nx, ny, nz = (int(v) for v in n)
    h = (hi - lo) / np.array([nx, ny, nz], dtype=np.float64)
    # lattice: fine units = half a coarse cell
    kz = np.arange(nz)
    zc = lo[2] + (kz + 0.5) * h[2]
    refine_layer = (np.abs(zc - lo[2]) < refine_band) | (np.abs(hi[2] - zc) < refine_band)
    if refine_cells is not None:  # explicit per-cell flags of the n-grid, x fastest
        refine_cells = np.asarray(refine_cells).reshape(nz, ny, nx) > 0
    cell_list = []  # (corner lattice coord (3,), size in fine units)
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                base = np.array([2 * i, 2 * j, 2 * k])
                if (refine_cells[k, j, i] if refine_cells is not None else refine_layer[k]):
                    for dk in range(2):
                        for dj in range(2):
                            for di in range(2):
                                cell_list.append((base + np.array([di, dj, dk]), 1))
                else:
                    cell_list.append((base, 2))
    corners = np.array([c for c, _ in cell_list], dtype=np.int64)
    sizes = np.array([s for _, s in cell_list], dtype=np.int64)
    offs = np.array([[(v >> 0) & 1, (v >> 1) & 1, (v >> 2) & 1] for v in range(8)], dtype=np.int64)
    vert = corners[:, None, :] + offs[None, :, :] * sizes[:, None, None]  # (nc, 8, 3)
    L = np.array([2 * nx + 1, 2 * ny + 1, 2 * nz + 1], dtype=np.int64)
    key = (vert[..., 2] * L[1] + vert[..., 1]) * L[0] + vert[..., 0]
    ukey, inv = np.unique(key.ravel(), return_inverse=True)
    cells = inv.reshape(-1, 8).astype(np.int32)
    # order cells by (z, y, x) of their first vertex lattice coordinate
    ckey = (corners[:, 2] * L[1] + corners[:, 1]) * L[0] + corners[:, 0]
    order = np.argsort(ckey, kind="stable")
    cells = cells[order]
    sizes = sizes[order]
    corners = corners[order]
    lat = np.stack([ukey % L[0], (ukey // L[0]) % L[1], ukey // (L[0] * L[1])], axis=1)
    xyz = lo[None, :] + lat * (h[None, :] * 0.5)
    nn = lat.shape[0]
    node_of = {int(k): idx for idx, k in enumerate(ukey)}

    def nid(p):
        return node_of.get(int((p[2] * L[1] + p[1]) * L[0] + p[0]), -1)

    # hanging nodes: on faces of coarse (size-2) cells, fine nodes at odd offsets
    parents = {}
    for c in range(cells.shape[0]):
        if sizes[c] != 2:
            continue
        b = corners[c]
        for axis in range(3):
            for side in range(2):
                # face of this coarse cell perpendicular to `axis`
                ta, tb = [a for a in range(3) if a != axis]
                for u in range(3):
                    for v in range(3):
                        if u != 1 and v != 1:
                            continue  # face corners are coarse vertices
                        p = b.copy()
                        p[axis] += 2 * side
                        p[ta] += u
                        p[tb] += v
                        n_id = nid(p)
                        if n_id < 0 or n_id in parents:
                            continue
                        if u == 1 and v == 1:
                            par = []
                            for uu in (0, 2):
                                for vv in (0, 2):
                                    q = b.copy()
                                    q[axis] += 2 * side
                                    q[ta] += uu
                                    q[tb] += vv
                                    par.append(nid(q))
                            parents[n_id] = (par, [0.25] * 4)
                        else:
                            q1 = p.copy()
                            q2 = p.copy()
                            if u == 1:
                                q1[ta] -= 1
                                q2[ta] += 1
                            else:
                                q1[tb] -= 1
                                q2[tb] += 1
                            parents[n_id] = ([nid(q1), nid(q2)], [0.5, 0.5])
    if periodic_x or periodic_y:
        # each node of an upper periodic face -> its image on the lower face (weight 1),
        # replacing a hanging constraint there; then substitute constrained parents until
        # all parents are unconstrained
        con = {k: list(zip(p, w)) for k, (p, w) in parents.items()}
        for axis, on in ((0, periodic_x), (1, periodic_y)):
            if not on:
                continue
            for idx in np.nonzero(lat[:, axis] == L[axis] - 1)[0]:
                q = lat[idx].copy()
                q[axis] = 0
                img = nid(q)
                assert img >= 0, "periodic image missing"
                con[int(idx)] = [(img, 1.0)]
        changed = True
        while changed:
            changed = False
            for k in list(con):
                acc = {}
                for p, w in con[k]:
                    if p in con:
                        changed = True
                        for pp, ww in con[p]:
                            acc[pp] = acc.get(pp, 0.0) + w * ww
                    else:
                        acc[p] = acc.get(p, 0.0) + w
                con[k] = sorted(acc.items())
        parents = {k: ([p for p, _ in t], [w for _, w in t]) for k, t in con.items()}
    hptr = np.zeros(nn + 1, dtype=np.int32)
    for n_id, (par, _) in parents.items():
        hptr[n_id + 1] = len(par)
    hptr = np.cumsum(hptr).astype(np.int32)
    hpar = np.zeros(hptr[-1], dtype=np.int32)
    hw = np.zeros(hptr[-1], dtype=np.float64)
    for n_id, (par, w) in parents.items():
        hpar[hptr[n_id]:hptr[n_id + 1]] = sorted(par)
        hw[hptr[n_id]:hptr[n_id + 1]] = w
    assert (hpar >= 0).all()
    mask = np.zeros(nn, dtype=np.uint32)
    hanging = np.diff(hptr) > 0
    for axis, on in ((0, dirichlet_x), (1, dirichlet_y), (2, dirichlet_z)):
        if not on:
            continue
        onface = (lat[:, axis] == 0) | (lat[:, axis] == L[axis] - 1)
        mask[onface & ~hanging] |= np.uint32(COLUMN_MASK[axis])
    return Mesh(xyz=xyz, cells=cells, mask=mask, hptr=hptr, hpar=hpar, hw=hw)


def cube_mesh(half: float, n: int, refine_frac: float = 0.0) -> Mesh:
    """The reference's cube [-half, half]^3 with n^3 cells, z faces pair-breaking."""
    return box_mesh([-half] * 3, [half] * 3, (n, n, n), refine_band=refine_frac * 2 * half)


@dataclasses.dataclass
class Mesh2D:
    xy: np.ndarray  # (nn, 2)
    cells: np.ndarray  # (nc, 4), vertex order v = ix + 2 iy
    mask: np.ndarray  # (nn,) uint32, bit c: component c zero-Dirichlet (2 components)

    @property
    def nn(self) -> int:
        return int(self.xy.shape[0])


def square_mesh(n: int, L: float = 1.0) -> Mesh2D:
    """Square [0, L]^2, n x n Q1 quads, psi = 0 (both components) on the x = 0 edge."""
    t = np.linspace(0.0, L, n + 1)
    X, Y = np.meshgrid(t, t, indexing="xy")
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    n0 = (j * (n + 1) + i).ravel()
    cells = np.stack([n0, n0 + 1, n0 + n + 1, n0 + n + 2], axis=1).astype(np.int32)
    mask = np.where(np.isclose(xy[:, 0], 0.0), 3, 0).astype(np.uint32)
    return Mesh2D(xy=xy, cells=cells, mask=mask)
