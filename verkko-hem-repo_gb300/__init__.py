"""GB300-native (sm_103a) femgl Newton hot path.

The product is ``lib/libglgpu.so`` (C ABI, ``include/glgpu.h``); ``glgpu`` is its
ctypes binding, shaped like the reference's FemGL members, and ``build`` compiles
it in-tree.  The directory name is not a Python identifier, so import it with
``importlib.import_module("verkko-hem-repo_gb300")``.
"""
from . import build as build_mod  # noqa: F401
from .glgpu import (FP64, MIXED, PC_BLOCK_JACOBI, PC_CHEBYSHEV, PC_MULTIGRID, PC_NONE, FemGL, GLGPUError, Mesh, Params, Surrogate,  # noqa: F401
                    bphase_guess, box_interpolate, box_mesh, box_mesh_refine, cube_mesh, lib, matep, mem_info, pdw_guess, pinned_array, plan_info, plan_kelly, plan_pattern, plan_prolongation, set_launch_mode,
                    plan_robin,
                    square_mesh)


def build(verbose: bool = False, force: bool = False) -> str:
    return build_mod.build(verbose=verbose, force=force)
