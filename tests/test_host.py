"""CPU tests of the product's host side: the C-ABI library loads and exports every
declared symbol, material parameters are bit-identical to the reference's, the box
mesher and the block pattern agree with the oracle's independent ones."""
import json
import os
import re

import numpy as np
import pytest

from _lib import ROOT, oracle_mesh, product

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def gl():
    return product()


def test_library_exports_every_declared_symbol(gl):
    header = open(os.path.join(ROOT, "include", "glgpu.h")).read()
    declared = set(re.findall(r"\b(glgpu_[a-z_]+)\s*\(", header))
    assert len(declared) >= 25
    L = gl.lib()
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing
    assert L.glgpu_version().decode().startswith("glgpu")


def test_matep_bit_identical_to_reference(gl):
    d = json.load(open(os.path.join(GOLD, "matep.json")))
    fields = d["fields"]
    for row in d["rows"]:
        got = gl.matep(row["p"], row["t"], bool(row["scc"]))
        for f, ref in zip(fields, row["out"]):
            assert got[f] == ref, (row["p"], row["t"], row["scc"], f, got[f], ref)


def test_matep_rejects_pressure_outside_table(gl):
    with pytest.raises(gl.GLGPUError):
        gl.matep(34.0, 0.5)
    with pytest.raises(gl.GLGPUError):
        gl.matep(-0.1, 0.5)


@pytest.mark.parametrize("n,frac", [(3, 0.0), (4, 0.25), (6, 1.0 / 6.0)])
def test_box_mesh_matches_oracle_mesher(gl, n, frac):
    from oracle import mesh as om

    p = gl.cube_mesh(10.0, n, frac)
    o = om.cube_mesh(10.0, n, frac)
    assert np.array_equal(p.cells, o.cells)
    assert np.allclose(p.xyz, o.xyz, rtol=0, atol=1e-12)
    assert np.array_equal(p.mask, o.mask)
    assert np.array_equal(p.hptr, o.hptr)
    assert np.array_equal(p.hpar, o.hpar)
    assert np.allclose(p.hw, o.hw)


def test_refined_cube_sizes_match_literal_geometry(gl):
    """64^3 cube, cells within 0.1 L of a z face refined once: 6 fine layers per side."""
    m = gl.cube_mesh(10.0, 64, 0.1)
    assert (m.nn, m.nc, m.n_hanging) == (648141, 606208, 24832)
    # hanging weights: 1/2 on edges, 1/4 on faces, always summing to 1
    w = np.add.reduceat(m.hw, m.hptr[:-1][np.diff(m.hptr) > 0])
    assert np.allclose(w, 1.0)


def test_z_faces_pair_breaking_mask(gl):
    m = gl.cube_mesh(10.0, 4)
    zmask = sum(1 << (9 * p + 3 * mu + 2) for p in range(2) for mu in range(3))
    onz = np.isclose(np.abs(m.xyz[:, 2]), 10.0)
    assert np.all(m.mask[onz] == zmask)
    assert np.all(m.mask[~onz] == 0)


@pytest.mark.parametrize("n,frac", [(4, 0.0), (4, 0.25)])
def test_block_pattern_matches_oracle(gl, oracle_gl, n, frac):
    m = gl.cube_mesh(10.0, n, frac)
    rowptr, cols = gl.plan_pattern([m])
    sysr = oracle_gl.System(oracle_mesh(m), np.zeros(8))
    assert np.array_equal(rowptr, sysr.rowptr)
    assert np.array_equal(cols, sysr.cols)


def test_plan_sizes_config_32cube(gl):
    info = gl.plan_info([gl.cube_mesh(10.0, 32)])
    assert info["n_nodes"] == 35937
    assert info["nnzb"] == 912673  # 97^3 node pairs
    assert info["max_row_blocks"] == 27


def test_batched_plan_concatenates(gl):
    a, b = gl.cube_mesh(10.0, 3), gl.cube_mesh(5.0, 4, 0.25)
    ia, ib, iab = gl.plan_info([a]), gl.plan_info([b]), gl.plan_info([a, b])
    assert iab["n_nodes"] == ia["n_nodes"] + ib["n_nodes"]
    assert iab["nnzb"] == ia["nnzb"] + ib["nnzb"]


def test_invalid_meshes_rejected(gl):
    m = gl.cube_mesh(10.0, 2)
    bad = gl.Mesh(3, m.xyz.copy(), m.cells.copy(), m.mask.copy())
    bad.cells[0, 0] = m.nn + 5
    with pytest.raises(gl.GLGPUError):
        gl.plan_info([bad])
    skew = gl.Mesh(3, m.xyz.copy(), m.cells.copy(), m.mask.copy())
    skew.xyz[skew.cells[0, 7], 0] += 0.3
    with pytest.raises(gl.GLGPUError):
        gl.plan_info([skew])


def test_bphase_guess(gl):
    x = gl.bphase_guess(20.0, 0.6, 5).reshape(5, 18)
    g = gl.matep(20.0, 0.6)["gap_B"] * float(np.float32(0.577350269))
    assert np.all(x[:, [0, 4, 8]] == g)
    assert np.all(x[:, [1, 2, 3, 5, 6, 7]] == 0) and np.all(x[:, 9:] == 0)
    y = gl.bphase_guess(20.0, 0.6, 5, noise=0.05, seed=2).reshape(5, 18)
    z = gl.bphase_guess(20.0, 0.6, 5, noise=0.05, seed=2).reshape(5, 18)
    assert np.array_equal(y, z) and 0.0 < np.std(y - x) < 0.2


@pytest.mark.parametrize("dxy,frac", [((0, 0), 0.0), ((0, 0), 0.25), ((1, 1), 0.3), ((1, 0), 0.0)])
def test_robin_faces_match_oracle(gl, oracle_gl, dxy, frac):
    """Pair-breaking (Robin) faces: the plan's classification equals the oracle's, including
    refined faces whose hanging nodes sit on the boundary."""
    m = gl.box_mesh([-1.0, -1.5, -1.25], [1.0, 1.5, 1.25], (4, 5, 4), refine_band=frac * 2.5, dirichlet_xy=dxy)
    bits = gl.plan_robin([m])
    ref = oracle_gl.System(oracle_mesh(m), np.zeros(9)).robin_faces()
    assert np.array_equal(bits, ref)
    # faces counted by geometry: every boundary face of a masked axis, nothing else
    lo, hi = m.xyz.min(0), m.xyz.max(0)
    expect = 0
    for e in range(m.nc):
        v = m.xyz[m.cells[e]]
        for ax, on in ((0, dxy[0]), (1, dxy[1]), (2, 1)):
            if on:
                for side, plane in ((0, lo[ax]), (1, hi[ax])):
                    on_face = [(vv >> ax) & 1 == side for vv in range(8)]
                    expect += int(np.all(v[on_face, ax] == plane))
    assert sum(bin(int(b)).count("1") for b in bits) == expect > 0
    if frac > 0:
        assert m.n_hanging > 0


def test_robin_bt_must_be_positive(gl):
    m = gl.cube_mesh(1.0, 2)
    with pytest.raises(gl.GLGPUError, match="bt"):
        gl.FemGL(m, gl.Params.from_matep(20.0, 0.6, bt=0.0))


@pytest.mark.parametrize("per,frac,dxy", [((1, 1), 0.0, (0, 0)), ((1, 0), 0.25, (0, 1)), ((1, 1), 0.3, (0, 0)),
                                          ((0, 1), 0.0, (1, 0))])
def test_periodic_box_mesh_matches_oracle_mesher(gl, oracle_gl, per, frac, dxy):
    """Periodic x / y faces (makegrid_retangle-z-AdGR_xy-periodic.cc): the upper face's
    nodes are constrained to their images, chains through edges and hanging nodes resolved."""
    from oracle import mesh as om

    lo, hi, n = [-1.0, -1.5, -1.25], [1.0, 1.5, 1.25], (4, 3, 4)
    p = gl.box_mesh(lo, hi, n, refine_band=frac * 2.5, dirichlet_xy=dxy, periodic_xy=per)
    o = om.box_mesh(lo, hi, n, refine_band=frac * 2.5, dirichlet_x=bool(dxy[0]), dirichlet_y=bool(dxy[1]),
                    periodic_x=bool(per[0]), periodic_y=bool(per[1]))
    assert np.array_equal(p.cells, o.cells)
    assert np.array_equal(p.mask, o.mask)
    assert np.array_equal(p.hptr, o.hptr)
    assert np.array_equal(p.hpar, o.hpar)
    assert np.array_equal(p.hw, o.hw)
    # every constrained node's parents are unconstrained, weights sum to one, and the
    # upper periodic faces are all constrained to nodes off those faces
    con = np.diff(p.hptr) > 0
    assert not con[p.hpar].any()
    assert np.allclose(np.add.reduceat(p.hw, p.hptr[:-1][con]), 1.0)
    top = np.max(p.xyz, axis=0)
    for axis in range(2):
        if per[axis]:
            upper = p.xyz[:, axis] == top[axis]
            assert con[upper].all()
            assert not (p.xyz[p.hpar, axis] == top[axis]).any()
    # block pattern and Robin faces agree with the oracle's on the periodic mesh
    rowptr, cols = gl.plan_pattern([p])
    sysr = oracle_gl.System(oracle_mesh(p), np.zeros(9))
    assert np.array_equal(rowptr, sysr.rowptr) and np.array_equal(cols, sysr.cols)
    assert np.array_equal(gl.plan_robin([p]), sysr.robin_faces())


def test_periodic_and_pair_breaking_exclusive(gl):
    with pytest.raises(ValueError):
        gl.box_mesh([0, 0, 0], [1, 1, 1], (2, 2, 2), dirichlet_xy=(1, 0), periodic_xy=(1, 0))


def test_pdw_guess_matches_reference_function(gl, oracle_gl):
    """The weak-coupling PDW initial state equals the reference's PDWconfig (pdw_config.h),
    recorded in tests/golden/pdw.npz (and compared live where the reference is built)."""
    g = np.load(os.path.join(GOLD, "pdw.npz"))
    x = gl.pdw_guess(float(g["p"]), float(g["t"]), g["points"], float(g["u"]), float(g["half_D"]),
                     scc=bool(g["scc"])).reshape(-1, 18)
    ref = g["values"]
    assert gl.matep(float(g["p"]), float(g["t"]))["gap_B"] == float(g["gap"])
    assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.abs(ref[:, 9:]).max() == 0.0 and np.abs(ref[:, :9]).max() > 0
    R = oracle_gl.ref()
    if R is None:
        return
    rng = np.random.default_rng(5)
    for _ in range(32):
        half_D, u = rng.uniform(2, 20), rng.uniform(-1, 1)
        q = 3.141592653589793 / (1.7320508075688772 * 2.0 * half_D)
        pt = np.array([rng.uniform(-30, 30), rng.uniform(-30, 30), rng.uniform(-half_D, half_D)])
        out = np.zeros(18)
        R.ref_pdw_value(u, q, half_D, float(g["gap"]), *pt, out.ctypes.data_as(oracle_gl._dp))
        mine = gl.pdw_guess(float(g["p"]), float(g["t"]), pt[None, :], u, half_D).reshape(18)
        assert np.abs(mine - out).max() <= 1e-12 * max(1.0, np.abs(out).max())


@pytest.mark.parametrize("per", [(0, 0), (1, 1)])
def test_refined_box_mesh_matches_oracle_mesher(gl, oracle_gl, per):
    """Cells chosen by flags refined once (the host half of adaptive refinement)."""
    from oracle import mesh as om

    lo, hi, n = [-1.0, -1.5, -1.25], [1.0, 1.5, 1.25], (4, 3, 4)
    flags = np.zeros(np.prod(n), np.int8)
    rng = np.random.default_rng(3)
    if per == (0, 0):
        flags[rng.choice(flags.size, 9, replace=False)] = 1
    else:  # periodic faces need matching refinement: refine whole z layers
        flags.reshape(n[2], n[1], n[0])[1] = 1
    p = gl.box_mesh_refine(lo, hi, n, flags, periodic_xy=per)
    o = om.box_mesh(lo, hi, n, refine_cells=flags, periodic_x=bool(per[0]), periodic_y=bool(per[1]))
    for f in ("cells", "mask", "hptr", "hpar", "hw"):
        assert np.array_equal(getattr(p, f), getattr(o, f)), f
    assert p.nc == np.prod(n) + 7 * int(flags.sum())
    rowptr, cols = gl.plan_pattern([p])
    sysr = oracle_gl.System(oracle_mesh(p), np.zeros(9))
    assert np.array_equal(rowptr, sysr.rowptr) and np.array_equal(cols, sysr.cols)
    if per == (1, 1):
        return
    # refinement that differs across periodic faces is refused
    with pytest.raises(gl.GLGPUError, match="periodic"):
        f2 = np.zeros(np.prod(n), np.int8)
        f2[0] = 1
        gl.box_mesh_refine(lo, hi, n, f2, periodic_xy=(1, 0))


def test_box_interpolate_is_trilinear(gl):
    lo, hi, n = [-1.0, -2.0, 0.0], [1.0, 2.0, 3.0], (2, 4, 3)
    coarse = gl.box_mesh(lo, hi, n)
    rng = np.random.default_rng(1)
    A = rng.standard_normal((18, 3))
    b = rng.standard_normal(18)
    xc = (coarse.xyz @ A.T + b).ravel()  # a linear field is reproduced exactly
    flags = np.ones(np.prod(n), np.int8)
    fine = gl.box_mesh_refine(lo, hi, n, flags)
    xf = gl.box_interpolate(lo, hi, n, xc, fine.xyz)
    assert np.allclose(xf, (fine.xyz @ A.T + b).ravel(), rtol=0, atol=1e-12)
    # nodes of the coarse grid keep their values exactly
    xn = gl.box_interpolate(lo, hi, n, rng.standard_normal(xc.size), coarse.xyz)
    xr = gl.box_interpolate(lo, hi, n, xn, coarse.xyz)
    assert np.array_equal(xn, xr)


def test_oracle_kelly_basic_properties():
    """The estimator's restatement: zero for a linear field, symmetric under mirror images,
    and fixed-number flags pick the largest estimates."""
    from oracle import kelly as ok
    from oracle import mesh as om

    lo, hi, n = [0.0, 0.0, 0.0], [2.0, 2.0, 2.0], (4, 4, 4)
    m = om.box_mesh(lo, hi, n, refine_band=0.6)
    x = np.tile(m.xyz @ np.array([0.3, -0.2, 0.7]), (18, 1)).T.ravel()
    assert np.abs(ok.kelly(m, x, lo, hi, n)).max() < 1e-12
    # a kink across the plane x = 1: only the cells touching it see a jump
    x = np.tile(np.abs(m.xyz[:, 0] - 1.0), (18, 1)).T.ravel()
    eta = ok.kelly(m, x, lo, hi, n)
    xc = m.xyz[m.cells].mean(axis=1)[:, 0]
    touch = (m.xyz[m.cells][:, :, 0] == 1.0).any(axis=1)
    assert np.all(eta[touch] > 0) and np.all(eta[~touch] < 1e-12)
    assert np.allclose(np.sort(eta[xc < 1]), np.sort(eta[xc > 1]))
    f = ok.fixed_number_flags(eta, 0.3)
    assert f.sum() >= int(0.3 * m.nc) and eta[f == 1].min() >= eta[f == 0].max()


@pytest.mark.parametrize("kind", ["band", "periodic", "periodic_band", "flags"])
def test_estimator_face_pairs_match_oracle(gl, kind):
    """The product's face pairing (node keys) equals the oracle's (point location)."""
    from oracle import kelly as ok

    lo, hi, n = [-2.0, -2.5, -1.5], [2.0, 2.5, 1.5], (4, 5, 3)
    per = (1, 1) if kind.startswith("periodic") else (0, 0)
    if kind == "flags":
        flags = np.zeros(np.prod(n), np.int8)
        flags[np.random.default_rng(8).choice(flags.size, 17, replace=False)] = 1
        m = gl.box_mesh_refine(lo, hi, n, flags)
    else:
        m = gl.box_mesh(lo, hi, n, refine_band=0.9 if "band" in kind else 0.0, periodic_xy=per)
    a, fa, b, fb, sub = gl.plan_kelly([m])
    mine = set()
    for k in range(a.size):
        if sub[k]:
            mine.add((int(a[k]), int(fa[k]), int(b[k]), 1))
        else:
            lo_c, hi_c = sorted((int(a[k]), int(b[k])))
            mine.add((lo_c, int(fa[k]) if a[k] < b[k] else int(fb[k]), hi_c, 0))
        assert fa[k] // 2 == fb[k] // 2 and fa[k] != fb[k]
    _, ref = ok.kelly(oracle_mesh(m), np.zeros(18 * m.nn), lo, hi, n, periodic=per, return_pairs=True)
    assert mine == ref


def _trilinear(x):
    return 1.5 + 0.3 * x[:, 0] - 0.7 * x[:, 1] + 0.2 * x[:, 2] + 0.05 * x[:, 0] * x[:, 1] * x[:, 2]


@pytest.mark.parametrize("kind", ["uniform", "band", "flags", "periodic_band", "periodic_flags", "batch"])
def test_multigrid_prolongation_reproduces_q1(gl, kind):
    """The first multigrid transfer: a once-refined box gets its unrefined grid as first coarse
    level, and P interpolates that grid's Q1 field at the fine nodes.  A trilinear field
    (periodic meshes: one of z only) on the coarse nodes comes back exactly at every free fine
    node; constrained fine nodes (hanging nodes, periodic images) have empty rows."""
    lo, hi, n = [-2.0, -2.5, -1.5], [2.0, 2.5, 1.5], (4, 5, 3)
    if kind == "uniform":
        meshes = [gl.box_mesh(lo, hi, n)]
    elif kind == "band":
        meshes = [gl.box_mesh(lo, hi, n, refine_band=0.9)]
    elif kind == "flags":
        flags = np.zeros(np.prod(n), np.int8)
        flags[np.random.default_rng(5).choice(flags.size, 11, replace=False)] = 1
        meshes = [gl.box_mesh_refine(lo, hi, n, flags)]
    elif kind == "periodic_band":
        meshes = [gl.box_mesh(lo, hi, n, refine_band=0.9, periodic_xy=(1, 1))]
    elif kind == "periodic_flags":
        # refined cells on both faces of each periodic axis (mirrored, as periodicity needs):
        # hanging nodes on the periodic faces resolve through the images
        flags = np.zeros(np.prod(n), np.int8)
        for i, j, k in ((0, 1, 1), (n[0] - 1, 1, 1), (2, 0, 0), (2, n[1] - 1, 0)):
            flags[(k * n[1] + j) * n[0] + i] = 1
        meshes = [gl.box_mesh_refine(lo, hi, n, flags, periodic_xy=(1, 1))]
    else:
        meshes = [gl.box_mesh(lo, hi, n, refine_band=0.9), gl.cube_mesh(2.0, 4)]
    out = gl.plan_prolongation(meshes)
    assert out is not None
    ptr, idx, w, xc = out
    xf = np.concatenate([np.asarray(m.xyz).reshape(-1, 3) for m in meshes])
    hp = np.concatenate([np.diff(np.asarray(m.hptr)) if m.hptr is not None else np.zeros(m.nn, int) for m in meshes])
    nco = xc.shape[0]
    if kind in ("band", "flags", "periodic_band", "periodic_flags"):
        assert nco == (n[0] + 1) * (n[1] + 1) * (n[2] + 1) and hp.sum() > 0
    f = (lambda x: 1.0 + 0.4 * x[:, 2]) if kind.startswith("periodic") else _trilinear
    rows = np.repeat(np.arange(ptr.size - 1), np.diff(ptr))
    Pf = np.bincount(rows, weights=w * f(xc)[idx], minlength=ptr.size - 1)
    free = hp == 0
    assert np.array_equal(np.diff(ptr) == 0, ~free)
    assert np.abs(Pf[free] - f(xf)[free]).max() <= 1e-12
    assert np.allclose(np.bincount(rows, weights=w, minlength=ptr.size - 1)[free], 1.0, atol=1e-14)
    assert idx.min() >= 0 and idx.max() < nco


def test_multigrid_prolongation_declines_l_shaped_domain(gl):
    """Cells of a box lattice that do not fill the box (an L-shaped domain) have no base grid:
    multigrid does not apply."""
    m = gl.box_mesh([0.0, 0.0, 0.0], [4.0, 4.0, 4.0], (4, 4, 4))
    cells = np.asarray(m.cells).reshape(-1, 8)
    xyz = np.asarray(m.xyz).reshape(-1, 3)
    lo_corner = xyz[cells[:, 0]]
    keep = ~((lo_corner[:, 0] >= 2.0) & (lo_corner[:, 1] >= 2.0))
    cells = cells[keep]
    used = np.unique(cells)
    renum = np.full(m.nn, -1, np.int64)
    renum[used] = np.arange(used.size)
    g = gl.Mesh(3, xyz[used], renum[cells].astype(np.int32), np.asarray(m.mask)[used])
    assert gl.plan_info([g])["n_nodes"] == used.size
    assert gl.plan_prolongation([g]) is None


def test_multigrid_prolongation_declines_graded_grid(gl):
    """A tensor grid with graded spacing is neither a uniform box grid nor a once-refined
    one: multigrid does not apply (the preconditioner falls back to block-Jacobi)."""
    m = gl.box_mesh([0.0, 0.0, 0.0], [4.0, 4.0, 4.0], (4, 4, 4))
    xyz = np.asarray(m.xyz).reshape(-1, 3).copy()
    xyz[:, 0] = xyz[:, 0] ** 2 / 4.0
    g = gl.Mesh(3, xyz, np.asarray(m.cells), np.asarray(m.mask))
    assert gl.plan_prolongation([m]) is not None
    assert gl.plan_prolongation([g]) is None


@pytest.mark.parametrize("kind", ["band", "flags", "periodic_band"])
def test_refined_galerkin_stays_in_base_pattern(gl, kind):
    """P^T J P of a once-refined box lies inside the block pattern of its unrefined grid (the
    first coarse level), checked on the block sparsity: a fine cell lies inside one base cell
    and a hanging node's parents are vertices of the base cell it borders."""
    import scipy.sparse as sp

    lo, hi, n = [-2.0, -2.5, -1.5], [2.0, 2.5, 1.5], (4, 5, 3)
    per = (1, 1) if kind == "periodic_band" else (0, 0)
    if kind == "flags":
        flags = np.zeros(np.prod(n), np.int8)
        flags[np.random.default_rng(9).choice(flags.size, 13, replace=False)] = 1
        m = gl.box_mesh_refine(lo, hi, n, flags)
    else:
        m = gl.box_mesh(lo, hi, n, refine_band=0.9, periodic_xy=per)
    base = gl.box_mesh(lo, hi, n, periodic_xy=per)
    ptr, idx, w, xc = gl.plan_prolongation([m])
    assert np.allclose(xc, np.asarray(base.xyz).reshape(-1, 3))
    rp, cols = gl.plan_pattern([m])
    crp, ccols = gl.plan_pattern([base])
    nf, nc = rp.size - 1, crp.size - 1
    S = sp.csr_matrix((np.ones(cols.size), cols, rp), shape=(nf, nf))
    P = sp.csr_matrix((np.ones(idx.size), idx, ptr), shape=(nf, nc))
    G = (P.T @ S @ P).tocoo()
    C = sp.csr_matrix((np.ones(ccols.size), ccols, crp), shape=(nc, nc))
    assert G.nnz > 0
    assert np.all(np.asarray(C[G.row, G.col]).ravel() > 0)


def test_oracle_start_and_coefficients_equal_the_product(gl, oracle_gl):
    """The CPU reference arm builds its workload from oracle code alone; its seeded
    B-phase start and its matep values must be the ones the GPU arm uses."""
    mp = oracle_gl.matep(20.0, 0.6)
    got = gl.matep(20.0, 0.6, True)
    for f in oracle_gl.MATEP_FIELDS:
        assert mp[f] == got[f], f
    for seed, noise in ((2, 0.05), (7, 0.0), (1000, 0.3)):
        a = oracle_gl.bphase_guess(mp["gap_B"], 777, noise, seed)
        b = gl.bphase_guess(20.0, 0.6, 777, noise=noise, seed=seed)
        assert np.array_equal(a, b), seed


def test_oracle_matep_table_lookup_rejects_untabulated_points(oracle_gl, monkeypatch):
    monkeypatch.setattr(oracle_gl, "ref", lambda: None)  # the GPU host has no compiled reference
    assert oracle_gl.matep(20.0, 0.6)["alpha"] == -0.4
    with pytest.raises(KeyError):
        oracle_gl.matep(20.5, 0.6)


_THREADS_SCRIPT = r"""
import hashlib, importlib, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
gl = importlib.import_module("verkko-hem-repo_gb300")
ms = [gl.box_mesh([-10, -10, -4], [10, 10, 4], (9, 9, 9)),
      gl.box_mesh([-6, -6, -6], [6, 6, 6], (8, 8, 8), refine_band=2.0),
      gl.box_mesh([-5, -5, -3], [5, 5, 3], (6, 6, 5), periodic_xy=(1, 1)),
      gl.box_mesh([-4, -4, -4], [4, 4, 4], (6, 6, 6), refine_band=1.5, periodic_xy=(1, 0))]
h = hashlib.sha256()
for a in (*gl.plan_pattern(ms), *gl.plan_prolongation(ms), *gl.plan_kelly(ms), gl.plan_robin(ms)):
    h.update(np.ascontiguousarray(a).tobytes())
sq = []
for nx, ny in ((40, 24), (9, 13)):
    X, Y = np.meshgrid(np.linspace(-1, 1, nx + 1), np.linspace(-1, 1, ny + 1))
    v0 = (np.arange(ny)[:, None] * (nx + 1) + np.arange(nx)[None, :]).ravel()
    cells = np.stack([v0, v0 + 1, v0 + nx + 1, v0 + nx + 2], 1).astype(np.int32)
    mask = ((np.abs(X) == 1) | (np.abs(Y) == 1)).ravel().astype(np.uint32)
    sq.append(gl.Mesh(2, np.stack([X.ravel(), Y.ravel()], 1), cells, mask))
for a in gl.plan_pattern(sq):
    h.update(np.ascontiguousarray(a).tobytes())
bad = gl.box_mesh([-1, -1, -1], [1, 1, 1], (4, 4, 4))
bad.cells[5, 3] = bad.nn + 7
skew = gl.box_mesh([-1, -1, -1], [1, 1, 1], (4, 4, 4))
skew.xyz[skew.cells[2, 7], 0] += 0.3
try:
    gl.plan_info([ms[0], skew, ms[2], bad])
    err = None
except gl.GLGPUError as e:
    err = str(e)
print(json.dumps({"info": gl.plan_info(ms), "hash": h.hexdigest(), "err": err}))
"""


def test_host_plans_do_not_depend_on_the_thread_count(gl):
    """The host builders split their work over instances and rows on all host threads; the
    block pattern, the multigrid prolongation (built with every level's plan, the transfer
    and the Galerkin tables), the estimator's face pairs and the Robin faces of a batch of
    plain, once-refined and periodic boxes, and the pattern of a batch of 2D meshes, are
    bitwise the same on 1 and 4 threads, and a batch with two invalid instances reports the
    first one."""
    import subprocess
    import sys
    out = []
    for threads in (1, 4):
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        r = subprocess.run([sys.executable, "-c", _THREADS_SCRIPT, ROOT], env=env, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        out.append(json.loads(r.stdout.strip().splitlines()[-1]))
    assert out[0] == out[1]
    assert "instance 1:" in out[0]["err"] and "axis-aligned box" in out[0]["err"]
