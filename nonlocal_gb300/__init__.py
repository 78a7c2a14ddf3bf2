"""GB300 (sm_103a) implementation of NonLocFEM's nonlocal thermal hot path.

The compute path is the CUDA library ``lib/libnlgpu.so`` (C ABI in
include/nlgpu.h, built by ``nonlocal_gb300.build``); ``thermal`` mirrors the
reference's solver API on top of it, ``meshgen`` makes structured meshes.
"""
from .meshgen import BILINEAR, SERENDIPITY, QuadMesh, read_su2, structured_quad_mesh, write_su2  # noqa: F401

__all__ = ["BILINEAR", "SERENDIPITY", "QuadMesh", "read_su2", "structured_quad_mesh", "write_su2"]
