"""ctypes binding of libglgpu.so, shaped like the reference's FemGL Newton interface.

The reference's path is a set of members of ``FemGL_mpi::FemGL<3>``
(femgl/inc/femgl.h:130-137): ``assemble_system()``, ``compute_residual()``,
``solve(tol)``, ``newton_iteration()`` and the ``run()`` loop that drives them.
:class:`FemGL` exposes the same calls with the same meaning, on a context that
holds one or more instances (meshes with their own coefficients).  Every call goes
through the C ABI declared in ``include/glgpu.h``; there is no other code path: if
the library cannot be loaded or the device is missing, the calls raise.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Sequence

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libglgpu.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_up = ctypes.POINTER(ctypes.c_uint32)
_lp = ctypes.POINTER(ctypes.c_int64)

FP64 = 0
MIXED = 1
PC_NONE = 0
PC_BLOCK_JACOBI = 1
PC_CHEBYSHEV = 2
PC_MULTIGRID = 3

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "not converged",
          5: "NaN/Inf", 6: "device wait timed out", 7: "call out of order"}
NOT_CONVERGED = 4

KERNEL_KINDS = ("spmv", "cell", "rows", "residual", "precond", "vector")
PHASES = ("assembly", "compute_residual", "solve", "newton_iteration")


class GLGPUError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"glgpu: {STATUS.get(status, status)}: {msg}")
        self.status = status


class _Mesh(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("n_nodes", ctypes.c_int), ("n_cells", ctypes.c_int), ("xyz", _dp),
                ("cells", _ip), ("dirichlet_mask", _up), ("hang_ptr", _ip), ("hang_parent", _ip),
                ("hang_weight", _dp)]


class _Params(ctypes.Structure):
    _fields_ = [("K1", ctypes.c_double), ("K2", ctypes.c_double), ("K3", ctypes.c_double),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double * 5), ("precision", ctypes.c_int),
                ("precond", ctypes.c_int), ("cheb_degree", ctypes.c_int), ("gmres_restart", ctypes.c_int),
                ("gmres_max_iter", ctypes.c_int), ("ls_step", ctypes.c_double), ("ls_max_trials", ctypes.c_int),
                ("damped", ctypes.c_int), ("mg_pre", ctypes.c_int), ("mg_post", ctypes.c_int),
                ("mg_omega", ctypes.c_double), ("mf_cells", ctypes.c_int), ("prec_reuse", ctypes.c_double),
                ("bt", ctypes.c_double), ("mg_coarse_shift", ctypes.c_double), ("mg_small_fuse", ctypes.c_int)]


_lib = None


def lib() -> ctypes.CDLL:
    """Load libglgpu.so (built by ``build.py``); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GLGPUError(1, f"{LIB_PATH} not built; run the package build first")
    L = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    L.glgpu_default_params.argtypes = [ctypes.POINTER(_Params)]
    L.glgpu_version.restype = ctypes.c_char_p
    L.glgpu_last_error.restype = ctypes.c_char_p
    L.glgpu_create.argtypes = [ctypes.POINTER(_Mesh), ctypes.POINTER(_Params), ctypes.c_int, ctypes.POINTER(vp)]
    L.glgpu_destroy.argtypes = [vp]
    L.glgpu_sizes.argtypes = [vp, _lp, _lp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.glgpu_set_solution.argtypes = [vp, _dp]
    L.glgpu_get_solution.argtypes = [vp, _dp]
    L.glgpu_assemble_system.argtypes = [vp, _dp]
    L.glgpu_compute_residual.argtypes = [vp, _dp]
    L.glgpu_solve.argtypes = [vp, ctypes.c_double, _ip]
    L.glgpu_newton_iteration.argtypes = [vp, _dp, _ip]
    L.glgpu_free_energy.argtypes = [vp, _dp]
    L.glgpu_run.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, _ip, _ip, _dp]
    L.glgpu_stop_norms.argtypes = [vp, _dp, _dp]
    L.glgpu_set_launch_mode.argtypes = [ctypes.c_int]
    L.glgpu_get_system.argtypes = [vp, _ip, _ip, _dp, _dp]
    L.glgpu_get_residual.argtypes = [vp, _dp]
    L.glgpu_get_update.argtypes = [vp, _dp]
    L.glgpu_spmv.argtypes = [vp, _dp, _dp]
    L.glgpu_timers.argtypes = [vp, _dp, ctypes.c_int]
    L.glgpu_kernel_timing.argtypes = [vp, ctypes.c_int, _dp, _lp, ctypes.c_int]
    L.glgpu_mg_levels.argtypes = [vp]
    L.glgpu_mg_fallbacks.argtypes = [vp]
    L.glgpu_mg_fallbacks.restype = ctypes.c_int64
    L.glgpu_set_mg_handoff.argtypes = [vp, ctypes.c_int]
    L.glgpu_mg_handed_off.argtypes = [vp, ctypes.POINTER(ctypes.c_uint8)]
    L.glgpu_set_reorthogonalization.argtypes = [vp, ctypes.c_int]
    L.glgpu_mg_level_info.argtypes = [vp, ctypes.c_int, _lp, _lp, _lp]
    L.glgpu_mg_level_system.argtypes = [vp, ctypes.c_int, _ip, _ip, _dp]
    L.glgpu_mg_prolongation.argtypes = [vp, ctypes.c_int, _ip, _ip, _dp]
    L.glgpu_mg_coarse_inverse.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)]
    L.glgpu_launch_count.argtypes = [vp]
    L.glgpu_launch_count.restype = ctypes.c_int64
    L.glgpu_device_bytes.argtypes = [vp]
    L.glgpu_device_bytes.restype = ctypes.c_int64
    L.glgpu_mem_info.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    L.glgpu_sync.argtypes = [vp]
    L.glgpu_event_start.argtypes = [vp]
    L.glgpu_event_stop.argtypes = [vp, _dp]
    L.glgpu_matep.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp]
    L.glgpu_mesh_box.argtypes = [_dp, _dp, _ip, ctypes.c_double, _ip, _ip, _ip, _ip, _dp, _ip, _up, _ip, _ip, _dp]
    L.glgpu_bphase_guess.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_uint64, _dp]
    L.glgpu_mesh_box_refine.argtypes = [_dp, _dp, _ip, ctypes.POINTER(ctypes.c_int8), _ip, _ip, _ip, _ip, _dp, _ip,
                                        _up, _ip, _ip, _dp]
    L.glgpu_box_interpolate.argtypes = [_dp, _dp, _ip, _dp, ctypes.c_int, _dp, _dp]
    L.glgpu_estimate_error.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
    L.glgpu_refine_flags.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_int8)]
    L.glgpu_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(vp)]
    L.glgpu_host_free.argtypes = [vp]
    L.glgpu_pdw_guess.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int, _dp, _dp]
    L.glgpu_dot_noalloc.argtypes = [vp, vp, ctypes.c_int64, vp, vp]
    fp = ctypes.POINTER(ctypes.c_float)
    L.glgpu_surrogate_create.argtypes = [ctypes.c_uint64, ctypes.POINTER(vp)]
    L.glgpu_surrogate_destroy.argtypes = [vp]
    L.glgpu_surrogate_set_normalization.argtypes = [vp, fp, fp]
    L.glgpu_surrogate_param_count.argtypes = [_lp]
    L.glgpu_surrogate_get_params.argtypes = [vp, fp]
    L.glgpu_surrogate_set_params.argtypes = [vp, fp]
    L.glgpu_surrogate_predict.argtypes = [vp, fp, ctypes.c_int, fp]
    L.glgpu_surrogate_gradient.argtypes = [vp, fp, fp, ctypes.c_int, fp, fp]
    L.glgpu_surrogate_train.argtypes = [vp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                        ctypes.c_uint64, fp]
    L.glgpu_surrogate_launch_count.argtypes = [vp]
    L.glgpu_surrogate_launch_count.restype = ctypes.c_int64
    L.glgpu_plan_info.argtypes = [ctypes.POINTER(_Mesh), ctypes.c_int, _lp]
    L.glgpu_plan_pattern.argtypes = [ctypes.POINTER(_Mesh), ctypes.c_int, _ip, _ip]
    L.glgpu_plan_robin.argtypes = [ctypes.POINTER(_Mesh), ctypes.c_int, ctypes.POINTER(ctypes.c_uint8)]
    _lib = L
    return L


def _check(status: int, allow: Sequence[int] = ()) -> int:
    if status != 0 and status not in allow:
        raise GLGPUError(status, lib().glgpu_last_error().decode())
    return status


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


# ---------------------------------------------------------------------------------
# host helpers
# ---------------------------------------------------------------------------------
MATEP_FIELDS = ("alpha", "beta1", "beta2", "beta3", "beta4", "beta5", "gap_A", "gap_B", "Tc_mK", "f_A", "f_B",
                "beta_A", "beta_B")


def matep(p: float, t: float, scc: bool = True) -> dict:
    """Material parameters at pressure p [bar] and t = T/Tc (reference matep)."""
    out = np.zeros(13)
    _check(lib().glgpu_matep(float(p), float(t), int(bool(scc)), _p(out)))
    return dict(zip(MATEP_FIELDS, out.tolist()))


@dataclasses.dataclass
class Mesh:
    dim: int
    xyz: np.ndarray
    cells: np.ndarray
    mask: np.ndarray
    hptr: np.ndarray | None = None
    hpar: np.ndarray | None = None
    hw: np.ndarray | None = None

    @property
    def nn(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def nc(self) -> int:
        return int(self.cells.shape[0])

    @property
    def n_hanging(self) -> int:
        return 0 if self.hptr is None else int(np.count_nonzero(np.diff(self.hptr)))

    def _struct(self) -> _Mesh:
        self.xyz = np.ascontiguousarray(self.xyz, np.float64)
        self.cells = np.ascontiguousarray(self.cells, np.int32)
        self.mask = np.ascontiguousarray(self.mask, np.uint32)
        s = _Mesh(self.dim, self.nn, self.nc, _p(self.xyz), _p(self.cells, _ip), _p(self.mask, _up), None, None, None)
        if self.hptr is not None and len(self.hpar) > 0:
            self.hptr = np.ascontiguousarray(self.hptr, np.int32)
            self.hpar = np.ascontiguousarray(self.hpar, np.int32)
            self.hw = np.ascontiguousarray(self.hw, np.float64)
            s.hang_ptr = _p(self.hptr, _ip)
            s.hang_parent = _p(self.hpar, _ip)
            s.hang_weight = _p(self.hw)
        return s


def box_mesh(lo, hi, n, refine_band: float = 0.0, dirichlet_xy=(0, 0), periodic_xy=(0, 0)) -> Mesh:
    """Box [lo, hi] with n cells per axis, z faces pair-breaking, cells within
    ``refine_band`` of a z face refined once (hanging nodes constrained).  x / y faces:
    pair-breaking where dirichlet_xy, periodic where periodic_xy, natural otherwise."""
    L = lib()
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    nv = np.asarray(n, np.int32)
    if any(d and p for d, p in zip(dirichlet_xy, periodic_xy)):
        raise ValueError("an axis is either pair-breaking or periodic")
    dxy = np.asarray([2 if p else (1 if d else 0) for d, p in zip(dirichlet_xy, periodic_xy)], np.int32)
    nn = ctypes.c_int()
    nc = ctypes.c_int()
    nh = ctypes.c_int()
    _check(L.glgpu_mesh_box(_p(lo), _p(hi), _p(nv, _ip), float(refine_band), _p(dxy, _ip), ctypes.byref(nn),
                            ctypes.byref(nc), ctypes.byref(nh), None, None, None, None, None, None))
    xyz = np.zeros((nn.value, 3))
    cells = np.zeros((nc.value, 8), np.int32)
    mask = np.zeros(nn.value, np.uint32)
    hptr = np.zeros(nn.value + 1, np.int32)
    hpar = np.zeros(max(nh.value, 1), np.int32)
    hw = np.zeros(max(nh.value, 1))
    _check(L.glgpu_mesh_box(_p(lo), _p(hi), _p(nv, _ip), float(refine_band), _p(dxy, _ip), ctypes.byref(nn),
                            ctypes.byref(nc), ctypes.byref(nh), _p(xyz), _p(cells, _ip), _p(mask, _up), _p(hptr, _ip),
                            _p(hpar, _ip), _p(hw)))
    return Mesh(3, xyz, cells, mask, hptr, hpar[:nh.value], hw[:nh.value])


def box_mesh_refine(lo, hi, n, flags, dirichlet_xy=(0, 0), periodic_xy=(0, 0)) -> Mesh:
    """The box [lo, hi] with n cells per axis and the cells with flags > 0 (cells of the
    unrefined grid, x fastest) refined once (hanging nodes constrained)."""
    L = lib()
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    nv = np.asarray(n, np.int32)
    f = np.ascontiguousarray(flags, np.int8)
    if f.size != int(np.prod(nv)):
        raise ValueError("one flag per cell of the unrefined grid")
    if any(d and p for d, p in zip(dirichlet_xy, periodic_xy)):
        raise ValueError("an axis is either pair-breaking or periodic")
    dxy = np.asarray([2 if p else (1 if d else 0) for d, p in zip(dirichlet_xy, periodic_xy)], np.int32)
    fp = f.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))
    nn, nc, nh = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(L.glgpu_mesh_box_refine(_p(lo), _p(hi), _p(nv, _ip), fp, _p(dxy, _ip), ctypes.byref(nn), ctypes.byref(nc),
                                   ctypes.byref(nh), None, None, None, None, None, None))
    xyz = np.zeros((nn.value, 3))
    cells = np.zeros((nc.value, 8), np.int32)
    mask = np.zeros(nn.value, np.uint32)
    hptr = np.zeros(nn.value + 1, np.int32)
    hpar = np.zeros(max(nh.value, 1), np.int32)
    hw = np.zeros(max(nh.value, 1))
    _check(L.glgpu_mesh_box_refine(_p(lo), _p(hi), _p(nv, _ip), fp, _p(dxy, _ip), ctypes.byref(nn), ctypes.byref(nc),
                                   ctypes.byref(nh), _p(xyz), _p(cells, _ip), _p(mask, _up), _p(hptr, _ip),
                                   _p(hpar, _ip), _p(hw)))
    return Mesh(3, xyz, cells, mask, hptr, hpar[:nh.value], hw[:nh.value])


def box_interpolate(lo, hi, n, x_box: np.ndarray, xyz: np.ndarray) -> np.ndarray:
    """Trilinear transfer of node values on the unrefined n-grid of [lo, hi] to points xyz."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    nv = np.asarray(n, np.int32)
    xb = np.ascontiguousarray(x_box, np.float64)
    xyz = np.ascontiguousarray(xyz, np.float64)
    out = np.zeros(18 * xyz.shape[0])
    _check(lib().glgpu_box_interpolate(_p(lo), _p(hi), _p(nv, _ip), _p(xb), int(xyz.shape[0]), _p(xyz), _p(out)))
    return out


def cube_mesh(half: float, n: int, refine_frac: float = 0.0) -> Mesh:
    """The reference's cube [-half, half]^3 (make_grid with "cube half side length")."""
    return box_mesh([-half] * 3, [half] * 3, (n, n, n), refine_band=refine_frac * 2.0 * half)


def square_mesh(n: int, L: float = 1.0) -> Mesh:
    """Square [0, L]^2, n x n Q1 quads, psi = 0 on the x = 0 edge (complexGL 2D;
    the archive's configuration is the unit square)."""
    t = np.linspace(0.0, L, n + 1)
    X, Y = np.meshgrid(t, t, indexing="xy")
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    n0 = (j * (n + 1) + i).ravel()
    cells = np.stack([n0, n0 + 1, n0 + n + 1, n0 + n + 2], axis=1).astype(np.int32)
    mask = np.where(np.isclose(xy[:, 0], 0.0), 3, 0).astype(np.uint32)
    return Mesh(2, xy, cells, mask)


class _Pinned:
    """Owner of a page-locked host allocation (freed when the last array view goes)."""

    def __init__(self, nbytes: int):
        self.ptr = ctypes.c_void_p()
        _check(lib().glgpu_host_alloc(int(nbytes), ctypes.byref(self.ptr)))

    def __del__(self):
        if getattr(self, "ptr", None) is not None and self.ptr.value:
            lib().glgpu_host_free(self.ptr)
            self.ptr = None


def mem_info():
    """(free, total) device memory in bytes."""
    fr, tot = ctypes.c_size_t(), ctypes.c_size_t()
    _check(lib().glgpu_mem_info(ctypes.byref(fr), ctypes.byref(tot)))
    return int(fr.value), int(tot.value)


def pinned_array(n: int, dtype=np.float64) -> np.ndarray:
    """A numpy array of n elements in page-locked host memory (direct DMA to and from the GPU)."""
    dt = np.dtype(dtype)
    owner = _Pinned(n * dt.itemsize)
    buf = (ctypes.c_char * (n * dt.itemsize)).from_address(owner.ptr.value)
    buf._owner = owner  # every view's base chain ends at buf, which keeps the allocation
    return np.frombuffer(buf, dtype=dt, count=n)


def pdw_guess(p: float, t: float, xyz: np.ndarray, u: float, half_D: float, scc: bool = True) -> np.ndarray:
    """Weak-coupling pair-density-wave start (B phase + modulation of amplitude u across a slab
    of thickness 2 half_D) at the node coordinates xyz [nn][3]."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    nn = xyz.shape[0]
    x = np.zeros(18 * nn)
    _check(lib().glgpu_pdw_guess(float(p), float(t), int(bool(scc)), float(u), float(half_D), int(nn), _p(xyz), _p(x)))
    return x


def set_launch_mode(programmatic: bool) -> None:
    """Programmatic dependent launch of the solve's kernels (default on); contexts created
    afterwards use the new mode."""
    _check(lib().glgpu_set_launch_mode(int(bool(programmatic))))


def bphase_guess(p: float, t: float, nn: int, noise: float = 0.0, seed: int = 0, scc: bool = True) -> np.ndarray:
    """B-phase start u11 = u22 = u33 = gap_B/sqrt(3) (+ seeded Gaussian noise)."""
    x = np.zeros(18 * nn)
    _check(lib().glgpu_bphase_guess(float(p), float(t), int(bool(scc)), int(nn), float(noise), int(seed), _p(x)))
    return x


def plan_info(meshes: Sequence[Mesh]) -> dict:
    """Host-only plan statistics of a list of instance meshes (no device needed)."""
    ms = (_Mesh * len(meshes))(*[m._struct() for m in meshes])
    info = np.zeros(6, np.int64)
    _check(lib().glgpu_plan_info(ms, len(meshes), _p(info, _lp)))
    keys = ("n_nodes", "nnzb", "max_row_blocks", "contributions", "hanging_targets", "segments")
    return dict(zip(keys, info.tolist()))


def plan_robin(meshes: Sequence[Mesh]) -> np.ndarray:
    """Host-only Robin face bits per cell (bit 2 axis + side), all instances concatenated."""
    ms = (_Mesh * len(meshes))(*[m._struct() for m in meshes])
    out = np.zeros(sum(m.nc for m in meshes), np.uint8)
    _check(lib().glgpu_plan_robin(ms, len(meshes), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
    return out


def plan_kelly(meshes: Sequence[Mesh]):
    """Host-only face pairs of the error estimator: arrays (a, fa, b, fb, sub)."""
    ms = (_Mesh * len(meshes))(*[m._struct() for m in meshes])
    L = lib()
    i8 = ctypes.POINTER(ctypes.c_int8)
    npairs = ctypes.c_int64()
    _check(L.glgpu_plan_kelly(ms, len(meshes), ctypes.byref(npairs), None, None, None, None, None))
    n = npairs.value
    a, b = np.zeros(n, np.int32), np.zeros(n, np.int32)
    fa, fb, sub = np.zeros(n, np.int8), np.zeros(n, np.int8), np.zeros(n, np.int8)
    _check(L.glgpu_plan_kelly(ms, len(meshes), ctypes.byref(npairs), _p(a, _ip), fa.ctypes.data_as(i8), _p(b, _ip),
                              fb.ctypes.data_as(i8), sub.ctypes.data_as(i8)))
    return a, fa, b, fb, sub


def plan_prolongation(meshes: Sequence[Mesh]):
    """Host-only multigrid prolongation from the first coarse level to the instance meshes:
    (ptr, idx, w, coarse_xyz) as node-level CSR over the fine nodes, or None when multigrid
    does not apply."""
    ms = (_Mesh * len(meshes))(*[m._struct() for m in meshes])
    L = lib()
    nco, nnz = ctypes.c_int64(), ctypes.c_int64()
    _check(L.glgpu_plan_prolongation(ms, len(meshes), ctypes.byref(nco), ctypes.byref(nnz), None, None, None, None))
    if nco.value == 0:
        return None
    ptr = np.zeros(sum(m.nn for m in meshes) + 1, np.int32)
    idx, w = np.zeros(nnz.value, np.int32), np.zeros(nnz.value)
    xyz = np.zeros((nco.value, 3))
    _check(L.glgpu_plan_prolongation(ms, len(meshes), ctypes.byref(nco), ctypes.byref(nnz), _p(ptr, _ip), _p(idx, _ip),
                                     _p(w, _dp), _p(xyz, _dp)))
    return ptr, idx, w, xyz


def plan_pattern(meshes: Sequence[Mesh]):
    """Host-only block pattern (rowptr, cols) of the condensed Jacobian."""
    info = plan_info(meshes)
    ms = (_Mesh * len(meshes))(*[m._struct() for m in meshes])
    rowptr = np.zeros(info["n_nodes"] + 1, np.int32)
    cols = np.zeros(info["nnzb"], np.int32)
    _check(lib().glgpu_plan_pattern(ms, len(meshes), _p(rowptr, _ip), _p(cols, _ip)))
    return rowptr, cols


@dataclasses.dataclass
class Params:
    """Coefficients and controls of one instance (see glgpu_params)."""
    alpha: float
    beta: Sequence[float] = (0.0, 0.0, 0.0, 0.0, 0.0)
    K1: float = 0.42072
    K2: float = 0.42072
    K3: float = 0.42072
    precision: int = FP64
    precond: int = PC_BLOCK_JACOBI
    cheb_degree: int = 3
    gmres_restart: int = 50
    gmres_max_iter: int = 10000
    ls_step: float = 0.83
    ls_max_trials: int = 100
    damped: bool = True
    mg_pre: int = 1
    mg_post: int = 1
    mg_omega: float = 1.0
    mf_cells: int = 8
    prec_reuse: float = 0.0
    #: "AdGR diffuse length": bt < 1e10 adds the Robin term (K1/bt) |A_t|^2 on the pair-breaking faces
    bt: float = 1e10
    #: multigrid: relative diagonal shift of the coarsest level's dense solve
    mg_coarse_shift: float = 1e-4
    #: multigrid, the small coarse levels: 0 one launch per sweep and transfer, 1 one cooperative
    #: launch per V-cycle, 2 one cluster launch per instance for the tail (True means 1)
    mg_small_fuse: int = 0

    @classmethod
    def from_matep(cls, p: float, t: float, scc: bool = True, **kw) -> "Params":
        m = matep(p, t, scc)
        return cls(alpha=m["alpha"], beta=[m[f"beta{i}"] for i in range(1, 6)], **kw)

    def _struct(self) -> _Params:
        s = _Params()
        lib().glgpu_default_params(ctypes.byref(s))
        s.K1, s.K2, s.K3, s.alpha = self.K1, self.K2, self.K3, self.alpha
        for i in range(5):
            s.beta[i] = float(self.beta[i]) if i < len(self.beta) else 0.0
        s.precision, s.precond, s.cheb_degree = int(self.precision), int(self.precond), int(self.cheb_degree)
        s.gmres_restart, s.gmres_max_iter = int(self.gmres_restart), int(self.gmres_max_iter)
        s.ls_step, s.ls_max_trials, s.damped = float(self.ls_step), int(self.ls_max_trials), int(bool(self.damped))
        s.mg_pre, s.mg_post, s.mg_omega = int(self.mg_pre), int(self.mg_post), float(self.mg_omega)
        s.mf_cells = int(self.mf_cells)
        s.prec_reuse = float(self.prec_reuse)
        s.bt = float(self.bt)
        s.mg_coarse_shift = float(self.mg_coarse_shift)
        s.mg_small_fuse = int(self.mg_small_fuse)
        return s


class FemGL:
    """One context: the Newton path of one or more instances on the GPU.

    Methods map one-to-one to the reference members they replace; vectors are the
    instances' node-major dof vectors concatenated in creation order."""

    def __init__(self, meshes: Mesh | Sequence[Mesh], params: Params | Sequence[Params]):
        L = lib()
        if isinstance(meshes, Mesh):
            meshes = [meshes]
        if isinstance(params, Params):
            params = [params] * len(meshes)
        if len(params) != len(meshes):
            raise ValueError("one Params per mesh")
        self.meshes = list(meshes)
        self._mstructs = (_Mesh * len(meshes))(*[m._struct() for m in meshes])
        self._pstructs = (_Params * len(meshes))(*[p._struct() for p in params])
        self._ctx = ctypes.c_void_p()
        _check(L.glgpu_create(self._mstructs, self._pstructs, len(meshes), ctypes.byref(self._ctx)))
        nn = ctypes.c_int64()
        nnzb = ctypes.c_int64()
        blk = ctypes.c_int()
        ni = ctypes.c_int()
        _check(L.glgpu_sizes(self._ctx, ctypes.byref(nn), ctypes.byref(nnzb), ctypes.byref(blk), ctypes.byref(ni)))
        self.n_nodes, self.nnzb, self.block, self.n_inst = nn.value, nnzb.value, blk.value, ni.value
        self.n_dofs = self.n_nodes * self.block
        offs = np.cumsum([0] + [m.nn for m in meshes])
        self.node_offsets = offs
        self.n_cells = int(sum(m.nc for m in meshes))

    # -- lifetime --
    def close(self) -> None:
        if getattr(self, "_ctx", None) is not None and self._ctx.value:
            lib().glgpu_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state --
    def set_solution(self, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        if x.size != self.n_dofs:
            raise ValueError(f"expected {self.n_dofs} dofs, got {x.size}")
        _check(lib().glgpu_set_solution(self._ctx, _p(x)))

    def solution(self, out: np.ndarray | None = None) -> np.ndarray:
        """The current solution (into `out` when given, e.g. a pinned_array)."""
        x = np.zeros(self.n_dofs) if out is None else out
        if x.dtype != np.float64 or x.size != self.n_dofs or not x.flags.c_contiguous:
            raise ValueError("out must be a contiguous float64 array of n_dofs entries")
        _check(lib().glgpu_get_solution(self._ctx, _p(x)))
        return x

    # -- the reference's members --
    def assemble_system(self) -> np.ndarray:
        out = np.zeros(self.n_inst)
        _check(lib().glgpu_assemble_system(self._ctx, _p(out)))
        return out

    def compute_residual(self) -> np.ndarray:
        out = np.zeros(self.n_inst)
        _check(lib().glgpu_compute_residual(self._ctx, _p(out)))
        return out

    def solve(self, tol: float, allow_unconverged: bool = False) -> np.ndarray:
        its = np.zeros(self.n_inst, np.int32)
        _check(lib().glgpu_solve(self._ctx, float(tol), _p(its, _ip)), (NOT_CONVERGED,) if allow_unconverged else ())
        return its

    def newton_iteration(self):
        res = np.zeros(self.n_inst)
        trials = np.zeros(self.n_inst, np.int32)
        _check(lib().glgpu_newton_iteration(self._ctx, _p(res), _p(trials, _ip)))
        return res, trials

    def run(self, max_newton: int = 40, linear_tol: float = 0.1, converge_acc: float = 5e-6,
            allow_unconverged: bool = False) -> dict:
        nits = np.zeros(self.n_inst, np.int32)
        gits = np.zeros(self.n_inst, np.int32)
        res = np.zeros(self.n_inst)
        st = _check(lib().glgpu_run(self._ctx, int(max_newton), float(linear_tol), float(converge_acc),
                                    _p(nits, _ip), _p(gits, _ip), _p(res)), (NOT_CONVERGED,) if allow_unconverged else ())
        ls = np.zeros(self.n_inst)
        r64 = np.zeros(self.n_inst)
        _check(lib().glgpu_stop_norms(self._ctx, _p(ls), _p(r64)))
        return {"newton_its": nits, "gmres_its": gits, "residual": res, "converged": st == 0,
                "residual_line_search": ls, "residual_fp64": r64}

    def free_energy(self) -> np.ndarray:
        out = np.zeros(self.n_inst)
        _check(lib().glgpu_free_energy(self._ctx, _p(out)))
        return out

    # -- inspection --
    def system(self):
        rowptr = np.zeros(self.n_nodes + 1, np.int32)
        cols = np.zeros(self.nnzb, np.int32)
        vals = np.zeros((self.nnzb, self.block, self.block))
        rhs = np.zeros(self.n_dofs)
        _check(lib().glgpu_get_system(self._ctx, _p(rowptr, _ip), _p(cols, _ip), _p(vals), _p(rhs)))
        return rowptr, cols, vals, rhs

    def residual(self) -> np.ndarray:
        R = np.zeros(self.n_dofs)
        _check(lib().glgpu_get_residual(self._ctx, _p(R)))
        return R

    def update(self) -> np.ndarray:
        d = np.zeros(self.n_dofs)
        _check(lib().glgpu_get_update(self._ctx, _p(d)))
        return d

    def spmv(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.n_dofs)
        _check(lib().glgpu_spmv(self._ctx, _p(x), _p(y)))
        return y

    # -- timing --
    def timers(self, reset: bool = False) -> dict:
        ms = np.zeros(4)
        _check(lib().glgpu_timers(self._ctx, _p(ms), int(reset)))
        return dict(zip(PHASES, ms.tolist()))

    def kernel_timing(self, enable, reset: bool = False):
        """enable: bitmask of kernel kinds to time (bit k = KERNEL_KINDS[k]); True = all."""
        ms = np.zeros(6)
        n = np.zeros(6, np.int64)
        mask = -1 if enable is True else int(enable)
        _check(lib().glgpu_kernel_timing(self._ctx, mask, _p(ms), _p(n, _lp), int(reset)))
        return dict(zip(KERNEL_KINDS, ms.tolist())), dict(zip(KERNEL_KINDS, n.tolist()))

    @property
    def launch_count(self) -> int:
        return int(lib().glgpu_launch_count(self._ctx))

    @property
    def device_bytes(self) -> int:
        """Device memory held by this context (multigrid levels included)."""
        return int(lib().glgpu_device_bytes(self._ctx))

    @property
    def mg_levels(self) -> int:
        return int(lib().glgpu_mg_levels(self._ctx))

    def mg_level(self, level: int):
        """(rowptr, cols, vals [nnzb][B][B], P as (ptr, idx, w)) of coarse level `level`."""
        L = lib()
        nn, nb, pn = np.zeros(1, np.int64), np.zeros(1, np.int64), np.zeros(1, np.int64)
        _check(L.glgpu_mg_level_info(self._ctx, int(level), _p(nn, _lp), _p(nb, _lp), _p(pn, _lp)))
        rowptr = np.zeros(nn[0] + 1, np.int32)
        cols = np.zeros(nb[0], np.int32)
        vals = np.zeros((nb[0], self.block, self.block))
        _check(L.glgpu_mg_level_system(self._ctx, int(level), _p(rowptr, _ip), _p(cols, _ip), _p(vals)))
        # prolongation rows are the nodes of the next finer level
        nf = self.n_nodes if level == 1 else int(self.mg_level_sizes(level - 1)[0])
        ptr = np.zeros(nf + 1, np.int32)
        idx = np.zeros(pn[0], np.int32)
        w = np.zeros(pn[0])
        _check(L.glgpu_mg_prolongation(self._ctx, int(level), _p(ptr, _ip), _p(idx, _ip), _p(w)))
        return rowptr, cols, vals, (ptr, idx, w)

    def mg_coarse_inverse(self, inst: int = 0) -> np.ndarray:
        """The coarsest level's dense FP32 inverse of instance `inst` (nd x nd) from the last
        preconditioner setup: (A + shift mean|diag A| I)^-1, the identity after a zero pivot."""
        L = lib()
        nd = ctypes.c_int(0)
        _check(L.glgpu_mg_coarse_inverse(self._ctx, int(inst), ctypes.byref(nd), None))
        inv = np.zeros((nd.value, nd.value), np.float32)
        _check(L.glgpu_mg_coarse_inverse(self._ctx, int(inst), ctypes.byref(nd),
                                         inv.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return inv

    def mg_level_sizes(self, level: int):
        nn, nb, pn = np.zeros(1, np.int64), np.zeros(1, np.int64), np.zeros(1, np.int64)
        _check(lib().glgpu_mg_level_info(self._ctx, int(level), _p(nn, _lp), _p(nb, _lp), _p(pn, _lp)))
        return int(nn[0]), int(nb[0]), int(pn[0])

    def estimate_error(self) -> np.ndarray:
        """Kelly error estimate per cell at the current solution (FP32, all instances)."""
        eta = np.zeros(self.n_cells, np.float32)
        _check(lib().glgpu_estimate_error(self._ctx, eta.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return eta

    def refine_flags(self, top_fraction: float, bottom_fraction: float = 0.0) -> np.ndarray:
        """Fixed-number refinement (1) / coarsening (-1) flags from the last estimate."""
        flags = np.zeros(self.n_cells, np.int8)
        _check(lib().glgpu_refine_flags(self._ctx, float(top_fraction), float(bottom_fraction),
                                        flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
        return flags

    @property
    def mg_fallbacks(self) -> int:
        return int(lib().glgpu_mg_fallbacks(self._ctx))

    def set_mg_handoff(self, on: bool = True) -> None:
        """Instances whose multigrid solve stalls twice stop at the state they reached in
        `run` (flagged in `handed_off`, reported unconverged) instead of finishing with
        block-Jacobi GMRES in this context."""
        _check(lib().glgpu_set_mg_handoff(self._ctx, int(bool(on))))

    def set_reorthogonalization(self, on: bool = True) -> None:
        """GMRES Gram-Schmidt with one reorthogonalization, or one projection (the default)."""
        _check(lib().glgpu_set_reorthogonalization(self._ctx, int(bool(on))))

    @property
    def handed_off(self) -> np.ndarray:
        """Per instance: handed off in the last `run`."""
        flags = np.zeros(self.n_inst, np.uint8)
        _check(lib().glgpu_mg_handed_off(self._ctx, flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return flags.astype(bool)

    def sync(self) -> None:
        _check(lib().glgpu_sync(self._ctx))

    def event_start(self) -> None:
        _check(lib().glgpu_event_start(self._ctx))

    def event_stop(self) -> float:
        ms = ctypes.c_double()
        _check(lib().glgpu_event_stop(self._ctx, ctypes.byref(ms)))
        return ms.value


_fp = ctypes.POINTER(ctypes.c_float)


class Surrogate:
    """The learned initial guess: an MLP (x, y, z, t, p, D) -> 256 x 4 (SiLU) -> 18 whose
    dense layers run on the tcgen05 tensor cores in BF16 with FP32 accumulation."""

    N_IN, N_OUT = 6, 18
    LAYERS = ((6, 256), (256, 256), (256, 256), (256, 256), (256, 18))

    def __init__(self, seed: int = 0):
        self._s = ctypes.c_void_p()
        _check(lib().glgpu_surrogate_create(int(seed), ctypes.byref(self._s)))
        n = ctypes.c_int64()
        _check(lib().glgpu_surrogate_param_count(ctypes.byref(n)))
        self.n_params = n.value

    def close(self):
        if getattr(self, "_s", None) is not None and self._s.value:
            lib().glgpu_surrogate_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_normalization(self, shift, scale):
        sh = np.ascontiguousarray(shift, np.float32)
        sc = np.ascontiguousarray(scale, np.float32)
        _check(lib().glgpu_surrogate_set_normalization(self._s, _p(sh, _fp), _p(sc, _fp)))

    def params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        _check(lib().glgpu_surrogate_get_params(self._s, _p(p, _fp)))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.n_params:
            raise ValueError("wrong parameter count")
        _check(lib().glgpu_surrogate_set_params(self._s, _p(p, _fp)))

    def predict(self, inputs) -> np.ndarray:
        x = np.ascontiguousarray(inputs, np.float32).reshape(-1, self.N_IN)
        y = np.zeros((x.shape[0], self.N_OUT), np.float32)
        _check(lib().glgpu_surrogate_predict(self._s, _p(x, _fp), x.shape[0], _p(y, _fp)))
        return y

    def gradient(self, inputs, targets):
        x = np.ascontiguousarray(inputs, np.float32).reshape(-1, self.N_IN)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, self.N_OUT)
        loss = ctypes.c_float()
        g = np.zeros(self.n_params, np.float32)
        _check(lib().glgpu_surrogate_gradient(self._s, _p(x, _fp), _p(t, _fp), x.shape[0], ctypes.byref(loss),
                                              _p(g, _fp)))
        return float(loss.value), g

    def train(self, inputs, targets, steps: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> float:
        x = np.ascontiguousarray(inputs, np.float32).reshape(-1, self.N_IN)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, self.N_OUT)
        loss = ctypes.c_float()
        _check(lib().glgpu_surrogate_train(self._s, _p(x, _fp), _p(t, _fp), x.shape[0], int(steps), int(batch),
                                           float(lr), int(seed), ctypes.byref(loss)))
        return float(loss.value)

    @property
    def launch_count(self) -> int:
        return int(lib().glgpu_surrogate_launch_count(self._s))
